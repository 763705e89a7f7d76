// renderer.cpp - Geometry, MatrixList, Drawable, StateSet and Renderer of
// the C++ facade (src/CadR/Drawable.cpp, StateSet.cpp, Renderer.cpp).
#include <CadR/Renderer.h>

#include <algorithm>
#include <chrono>
#include <cstddef>
#include <cstring>
#include <unordered_set>

namespace CadR {

Geometry::Geometry(Renderer& r)
    : _renderer(&r), _vertices(r.dataStorage()), _indices(r.dataStorage()), _primitiveSets(r.dataStorage())
{
}

MatrixList::MatrixList(Renderer& r) : _list(r.dataStorage()) {}

// Header {numMatrices, capacity, 7 x uint64 0} then the matrices
// (MatrixList.h:54-58).
void* MatrixList::newContent(size_t n)
{
    StagingData s = _list.alloc(64 + 64 * n);
    uint8_t* p = s.data<uint8_t>();
    std::memset(p, 0, 64);
    const uint32_t n32 = uint32_t(n);
    std::memcpy(p, &n32, 4);
    std::memcpy(p + 4, &n32, 4);
    return p + 64;
}

void MatrixList::setMatrixData(const void* m, size_t n)
{
    void* p = newContent(n);
    if (n) std::memcpy(p, m, 64 * n);
}

// ---------------------------------------------------------------------------
// Drawable (Drawable.cpp:35-78).

Drawable::Drawable(Geometry& g, uint32_t off, MatrixList& ml, StateSet& ss) { create(g, off, ml, nullptr, ss); }

Drawable::Drawable(Geometry& g, uint32_t off, MatrixList& ml, DataAllocation& dd, StateSet& ss)
{
    create(g, off, ml, &dd, ss);
}

void Drawable::create(Geometry& g, uint32_t off, MatrixList& ml, StateSet& ss) { create(g, off, ml, nullptr, ss); }

void Drawable::create(Geometry& g, uint32_t off, MatrixList& ml, DataAllocation& dd, StateSet& ss)
{
    create(g, off, ml, &dd, ss);
}

// The record of Drawable.cpp:35-78: geometry handles, MatrixList handle,
// drawable-data handle (0 without one), PrimitiveSet offset.
void Drawable::create(Geometry& g, uint32_t off, MatrixList& ml, DataAllocation* dd, StateSet& ss)
{
    destroy();
    _matrixList = &ml;
    _drawableData = dd;
    ss.append(*this, DrawableGpuData(g.vertexDataAllocation().handle(), g.indexDataAllocation().handle(), ml.handle(),
                                     dd ? dd->handle() : 0, g.primitiveSetDataAllocation().handle(), off));
}

Drawable::Drawable(Drawable&& o) noexcept
    : _stateSet(o._stateSet), _matrixList(o._matrixList), _drawableData(o._drawableData), _index(o._index)
{
    if (_index != ~0u) _stateSet->_drawables[_index] = this;
    o._index = ~0u;
}

Drawable& Drawable::operator=(Drawable&& o) noexcept
{
    if (this == &o) return *this;
    destroy();
    _stateSet = o._stateSet;
    _matrixList = o._matrixList;
    _drawableData = o._drawableData;
    _index = o._index;
    if (_index != ~0u) _stateSet->_drawables[_index] = this;
    o._index = ~0u;
    return *this;
}

Drawable::~Drawable() { destroy(); }

Renderer& Drawable::renderer() const { return _stateSet->renderer(); }

void Drawable::destroy() noexcept
{
    if (_index != ~0u) _stateSet->remove(*this);
}

// ---------------------------------------------------------------------------
// StateSet (StateSet.cpp:20-47,180-268).

// childList and parentList sit in a class that is not standard-layout;
// offsetof is supported for it by the compilers this builds with.
#pragma GCC diagnostic push
#pragma GCC diagnostic ignored "-Winvalid-offsetof"
const ParentChildListOffsets StateSet::parentChildListOffsets{offsetof(StateSet, parentList),
                                                              offsetof(StateSet, childList)};
#pragma GCC diagnostic pop

StateSet::~StateSet() { removeAllDrawables(); }

void StateSet::removeAllDrawables() noexcept
{
    for (Drawable* d : _drawables) d->_index = ~0u;
    for (uint32_t s : _slots) _renderer->freeSlot(s);
    _records.clear();
    _drawables.clear();
    _slots.clear();
}

void StateSet::appendDrawable(Drawable& d, const DrawableGpuData& g)
{
    if (d._index != ~0u) d._stateSet->remove(d);
    append(d, g);
}

void StateSet::removeDrawable(Drawable& d) noexcept
{
    if (d._index != ~0u) d._stateSet->remove(d);
}

void StateSet::removeChild(StateSet& child)
{
    for (auto it = childList.begin(); it != childList.end(); ++it)
        if (&*it == &child) {
            childList.remove(it);
            return;
        }
}

void StateSet::append(Drawable& d, const DrawableGpuData& g)
{
    d._stateSet = this;
    d._index = uint32_t(_records.size());
    _records.push_back(g);
    _drawables.push_back(&d);
    _slots.push_back(_renderer->allocSlot(this, g));
}

// O(1) removal: the last record takes the removed one's place.
void StateSet::remove(Drawable& d) noexcept
{
    const uint32_t i = d._index;
    const size_t last = _records.size() - 1;
    _renderer->freeSlot(_slots[i]);
    if (i != last) {
        _records[i] = _records[last];
        Drawable* moved = _drawables[last];
        _drawables[i] = moved;
        moved->_index = i;
        _slots[i] = _slots[last];
    }
    _records.pop_back();
    _drawables.pop_back();
    _slots.pop_back();
    d._index = ~0u;
}

size_t StateSet::prepareRecording()
{
    _skipRecording = !_forceRecording;
    for (auto& f : prepareCallList) f(*this);
    size_t n = _records.size();
    for (StateSet& c : childList) {
        n += c.prepareRecording();
        _skipRecording = _skipRecording && c._skipRecording;
    }
    _skipRecording = _skipRecording && n == 0;
    return n;
}

void StateSet::recordToCommandBuffer(std::vector<DrawCall>& out, size_t& counter)
{
    if (_skipRecording) return;
    const size_t n = _records.size();
    if (n > 0) {
        std::memcpy(_renderer->drawableStagingData() + counter, _records.data(), n * sizeof(DrawableGpuData));
        out.push_back(DrawCall{this, counter, uint32_t(n),
                               _renderer->drawablePointersBufferAddress() + counter * Renderer::drawablePointersRecordSize,
                               counter * sizeof(cadr_draw_indirect_cmd)});
        counter += n;
    }
    for (StateSet& c : childList) c.recordToCommandBuffer(out, counter);
}

void StateSet::recordDrawCalls(std::vector<DrawCall>& out, size_t& counter) const
{
    if (_skipRecording) return;
    const size_t n = _records.size();
    if (n > 0) {
        out.push_back(DrawCall{this, counter, uint32_t(n),
                               _renderer->drawablePointersBufferAddress() + counter * Renderer::drawablePointersRecordSize,
                               counter * sizeof(cadr_draw_indirect_cmd)});
        counter += n;
    }
    for (const StateSet& c : childList) c.recordDrawCalls(out, counter);
}

// ---------------------------------------------------------------------------
// Renderer.

Renderer* Renderer::_defaultRenderer = nullptr;

Renderer::Renderer(bool makeDefault) : Renderer(0, makeDefault) {}

Renderer::Renderer(int device, bool makeDefault)
{
    _ownBackend = std::make_unique<CudaMemoryBackend>(device);
    _backend = _ownBackend.get();
    _storage = std::make_unique<DataStorage>(*_backend);
    _storage->setRenderer(this);
    if (makeDefault) _defaultRenderer = this;
}

Renderer::Renderer(MemoryBackend& backend, bool makeDefault) : _backend(&backend)
{
    _storage = std::make_unique<DataStorage>(*_backend);
    _storage->setRenderer(this);
    if (makeDefault) _defaultRenderer = this;
}

Renderer::~Renderer()
{
    if (_defaultRenderer == this) _defaultRenderer = nullptr;
    finalize();
    _storage.reset();
    _ownBackend.reset();  // destroys the context this renderer created
}

void Renderer::finalize()
{
    if (cadr_context* c = _backend->existingContext()) cadr_context_synchronize(c);
    if (_pack) cadr_pack_destroy(_pack);
    if (_drawables) _backend->freeBlock(_drawables);
    if (_indirect) _backend->freeBlock(_indirect);
    if (_pointers) _backend->freeBlock(_pointers);
    leakResources();
}

void Renderer::leakResources() noexcept
{
    _pack = nullptr;
    _packCapacity = 0;
    _drawables = _indirect = _pointers = 0;
    _capacity = 0;
}

size_t Renderer::beginFrame()
{
    _frame++;
    _storage->setFrameNumber(_frame);
    // the previous frame's uploads become the staging size hint
    // (Renderer.cpp:394-397)
    _lastFrameUploadBytes = _currentFrameUploadBytes;
    _currentFrameUploadBytes = 0;
    _storage->setStagingDataSizeHint(_lastFrameUploadBytes);
    _currentInfo = FrameInfo{};
    _currentInfo.frameNumber = _frame;
    _currentInfo.cpuBeginFrame = getCpuTimestamp();
    _currentInfo.gpuBeginFrame = _currentInfo.cpuBeginFrame;
    _gpuStamps = 0;
    return _frame;
}

uint64_t Renderer::getCpuTimestamp() const
{
    return uint64_t(std::chrono::duration_cast<std::chrono::nanoseconds>(
                        std::chrono::steady_clock::now().time_since_epoch())
                        .count());
}

void Renderer::setCollectFrameInfo(bool on, bool /*useCalibratedTimestamps*/) { _collect = on; }

// GPU timestamp `index` of the current frame (FrameInfo's four GPU fields).
void Renderer::timestamp(uint32_t index, cadr_stream stream)
{
    if (!_collect) return;
    cadr_context* ctx = _backend->context();
    if (!ctx) return;
    if (index == 0) _currentInfo.gpuBeginExecution = getCpuTimestamp();
    check(cadr_context_record_timestamp(ctx, _frame, index, stream), "Renderer: frame timestamp");
    _gpuStamps |= 1u << index;
    _frameStream = stream;
}

void Renderer::endFrame()
{
    _currentInfo.cpuEndFrame = getCpuTimestamp();
    _endedHasGpu = false;
    if (_collect && _gpuStamps == 7u) {
        timestamp(3, _frameStream);
        _endedHasGpu = true;
        _endedGpuBase = _currentInfo.gpuBeginExecution;
    }
    _lastInfo = _currentInfo;
    _endedFrame = _frame;
}

const FrameInfo& Renderer::getFrameInfo()
{
    if (_endedFrame == ~size_t(0) || !_endedHasGpu) {
        _lastInfo.frameNumber = ~size_t(0);
        return _lastInfo;
    }
    uint64_t ns[4];
    check(cadr_context_read_timestamps(_backend->context(), _endedFrame, ns), "Renderer: frame timestamps");
    _lastInfo.frameNumber = _endedFrame;
    _lastInfo.gpuBeginExecution = _endedGpuBase + ns[0];
    _lastInfo.gpuAfterTransfersAndBeforeDrawableProcessing = _endedGpuBase + ns[1];
    _lastInfo.gpuAfterDrawableProcessingAndBeforeRendering = _endedGpuBase + ns[2];
    _lastInfo.gpuEndExecution = _endedGpuBase + ns[3];
    return _lastInfo;
}

// Buffer growth of Renderer::prepareSceneRendering (Renderer.cpp:461-592):
// 20% extra, at least 128 drawables.
void Renderer::growBuffers(size_t n)
{
    if (_capacity >= n) return;
    size_t cap = size_t(float(n) * 1.2f);
    if (cap < 128) cap = 128;
    if (cadr_context* c = _backend->existingContext()) cadr_context_synchronize(c);
    if (_drawables) _backend->freeBlock(_drawables);
    if (_indirect) _backend->freeBlock(_indirect);
    if (_pointers) _backend->freeBlock(_pointers);
    _drawables = _backend->allocBlock(cap * sizeof(DrawableGpuData));
    _indirect = _backend->allocBlock(cap * sizeof(cadr_draw_indirect_cmd));
    _pointers = _backend->allocBlock(cap * drawablePointersRecordSize);
    if (!_drawables || !_indirect || !_pointers) throw OutOfResources("Renderer: cannot allocate drawable buffers");
    _staging.assign(cap, DrawableGpuData{});
    _capacity = cap;
}

size_t Renderer::prepareSceneRendering(StateSet& root)
{
    _currentInfo.cpuPrepareRecordingBegin = getCpuTimestamp();
    const size_t n = root.prepareRecording();
    _currentInfo.cpuPrepareRecordingEnd = getCpuTimestamp();
    growBuffers(n);
    return n;
}

void Renderer::recordSceneRendering(StateSet& root, std::vector<DrawCall>& out)
{
    size_t counter = 0;
    _currentInfo.cpuRecordStateSetsBegin = getCpuTimestamp();
    root.recordToCommandBuffer(out, counter);
    _currentInfo.cpuRecordStateSetsEnd = getCpuTimestamp();
}

size_t Renderer::executeCopyOperations()
{
    const size_t bytes = _storage->uploadPending();
    _currentFrameUploadBytes += bytes;
    return bytes;
}

void Renderer::recordDrawableProcessing(size_t n, cadr_stream stream)
{
    if (n == 0) return;
    cadr_context* ctx = _backend->context();
    if (!ctx) throw LogicError("Renderer::recordDrawableProcessing(): this renderer has no CUDA context");
    if (n > _capacity) throw LogicError("Renderer::recordDrawableProcessing(): call prepareSceneRendering() first");
    if (!(_gpuStamps & 1u)) timestamp(0, stream);
    check(cadr_upload(ctx, reinterpret_cast<void*>(_drawables), _staging.data(), n * sizeof(DrawableGpuData), stream),
          "Renderer: drawable upload");
    timestamp(1, stream);
    check(cadr_process_drawables(ctx, _storage->handleLevel(), reinterpret_cast<const void*>(_storage->handleTableDeviceAddress()),
                                 reinterpret_cast<const cadr_drawable_gpu_data*>(_drawables), n,
                                 reinterpret_cast<cadr_draw_indirect_cmd*>(_indirect),
                                 reinterpret_cast<cadr_drawable_pointers*>(_pointers), stream),
          "Renderer: processDrawables");
    timestamp(2, stream);
}

void Renderer::processDrawables(StateSet& root, std::vector<DrawCall>& out, cadr_stream stream)
{
    const size_t n = prepareSceneRendering(root);
    recordSceneRendering(root, out);
    if (n) timestamp(0, stream);
    executeCopyOperations();
    recordDrawableProcessing(n, stream);
}

// ---------------------------------------------------------------------------
// Device-resident records.

uint32_t Renderer::allocSlot(StateSet* owner, const DrawableGpuData& g)
{
    uint32_t s;
    if (!_freeSlots.empty()) {
        s = _freeSlots.back();
        _freeSlots.pop_back();
        _slotOwner[s] = owner;
    } else {
        s = uint32_t(_slotOwner.size());
        _slotOwner.push_back(owner);
    }
    _newSlots.push_back(s);
    _newRecords.push_back(g);
    _layoutDirty = true;
    return s;
}

void Renderer::freeSlot(uint32_t s) noexcept
{
    _slotOwner[s] = nullptr;
    _freeSlots.push_back(s);
    _layoutDirty = true;
}

// A larger pack: every live record is queued again (from the StateSets'
// host lists, which stay authoritative).
void Renderer::growPack(uint32_t slots)
{
    cadr_context* ctx = _backend->context();
    const uint32_t cap = std::max<uint32_t>(1024u, uint32_t(slots + slots / 2));
    cadr_pack* p = nullptr;
    check(cadr_pack_create(ctx, cap, &p), "Renderer: pack");
    if (_pack) {
        cadr_context_synchronize(ctx);
        cadr_pack_destroy(_pack);
    }
    _pack = p;
    _packCapacity = cap;
    _newSlots.clear();
    _newRecords.clear();
    std::vector<bool> seen(_slotOwner.size(), false);
    for (uint32_t s = 0; s < _slotOwner.size(); s++) {
        StateSet* ss = _slotOwner[s];
        if (!ss || seen[s]) continue;
        for (size_t li = 0; li < ss->_slots.size(); li++) {
            seen[ss->_slots[li]] = true;
            _newSlots.push_back(ss->_slots[li]);
            _newRecords.push_back(ss->_records[li]);
        }
    }
    _layoutDirty = true;
}

void Renderer::processDrawablesResident(StateSet& root, std::vector<DrawCall>& out, cadr_stream stream)
{
    cadr_context* ctx = _backend->context();
    if (!ctx) throw LogicError("Renderer::processDrawablesResident(): this renderer has no CUDA context");
    // A StateSet reached twice (a child of two parents) is recorded twice,
    // which one slot per record cannot express: such a frame takes the
    // copying path.
    // The walk also lists the tree's StateSets in a fixed order: when the
    // list differs from the previous frame's (a child appended, removed or
    // moved), the pack is laid out again.
    {
        std::unordered_set<const StateSet*> seen;
        std::vector<const StateSet*> stack{&root}, tree;
        while (!stack.empty()) {
            const StateSet* ss = stack.back();
            stack.pop_back();
            if (!seen.insert(ss).second) {
                processDrawables(root, out, stream);
                return;
            }
            tree.push_back(ss);
            for (const StateSet& c : ss->childList) stack.push_back(&c);
        }
        if (tree != _tree) {
            _tree.swap(tree);
            _layoutDirty = true;
        }
    }
    const size_t n = prepareSceneRendering(root);
    size_t counter = 0;
    _currentInfo.cpuRecordStateSetsBegin = getCpuTimestamp();
    root.recordDrawCalls(out, counter);
    _currentInfo.cpuRecordStateSetsEnd = getCpuTimestamp();
    if (n) timestamp(0, stream);
    executeCopyOperations();
    const uint32_t slots = uint32_t(_slotOwner.size());
    if (slots > _packCapacity) growPack(slots);
    if (_layoutDirty) {
        // StateSets in recording order, depth-first from the root; every slot
        // not reached from it (free, or in a StateSet outside the tree) goes
        // to one trailing set that is never drawn.
        std::vector<uint32_t> setOf(slots, ~0u), indexOf(slots, 0);
        uint32_t id = 0;
        std::vector<const StateSet*> stack{&root};
        while (!stack.empty()) {
            const StateSet* ss = stack.back();
            stack.pop_back();
            for (size_t li = 0; li < ss->_slots.size(); li++) {
                setOf[ss->_slots[li]] = id;
                indexOf[ss->_slots[li]] = uint32_t(li);
            }
            id++;
            for (auto it = ss->childList.rbegin(); it != ss->childList.rend(); ++it) stack.push_back(&*it);
        }
        uint32_t rest = 0;
        for (uint32_t s = 0; s < slots; s++)
            if (setOf[s] == ~0u) {
                setOf[s] = id;
                indexOf[s] = rest++;
            }
        std::vector<uint32_t> dfs(id + 1);
        for (uint32_t k = 0; k <= id; k++) dfs[k] = k;
        check(cadr_pack_set_layout(_pack, slots, id + 1, dfs.data(), setOf.data(), indexOf.data(), stream),
              "Renderer: pack layout");
    }
    if (!_newSlots.empty()) {
        check(cadr_pack_patch(_pack, _newSlots.data(), reinterpret_cast<const cadr_drawable_gpu_data*>(_newRecords.data()),
                              uint32_t(_newSlots.size()), stream),
              "Renderer: new records");
        _newSlots.clear();
        _newRecords.clear();
    }
    _layoutDirty = false;
    if (n == 0) return;
    timestamp(1, stream);
    // processDrawables straight from the pool (slots in creation order), so
    // no repack is needed; the first n packed positions are the drawn ones.
    check(cadr_pack_process_drawables(_pack, _storage->handleLevel(),
                                      reinterpret_cast<const void*>(_storage->handleTableDeviceAddress()), uint32_t(n),
                                      reinterpret_cast<cadr_draw_indirect_cmd*>(_indirect),
                                      reinterpret_cast<cadr_drawable_pointers*>(_pointers), stream),
          "Renderer: processDrawables");
    timestamp(2, stream);
}

}  // namespace CadR
