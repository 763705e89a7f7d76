// CadR/Renderer.h - the scene objects and the frame driver of the C++
// facade: Geometry, PrimitiveSet, MatrixList, Drawable, StateSet, Renderer,
// with the reference's names, data layouts and recording order.
//
//   Geometry     three DataAllocations: vertices, indices, PrimitiveSets
//                (src/CadR/Geometry.h:37-39)
//   MatrixList   64-byte header {numMatrices, capacity, 0...} + mat4[n]
//                (src/CadR/MatrixList.h:54-59)
//   Drawable     one DrawableGpuData record in its StateSet's list
//                (src/CadR/Drawable.h:32-43, Drawable.cpp:35-78)
//   StateSet     per-StateSet record list with O(1) swap-remove, child and
//                parent lists (CadR/ParentChildList.h), prepareRecording /
//                recordToCommandBuffer in depth-first order
//                (src/CadR/StateSet.h:77-79, StateSet.cpp:20-47,180-268)
//   Renderer     buffer growth x1.2 (min 128), drawable processing through
//                cadr_process_drawables, uploads, frame timing
//                (src/CadR/Renderer.cpp:446-720,946-999)
//
// Difference from the reference: there is no deferred command buffer, so
// recordDrawableProcessing() runs the pass when called and must come after
// recordSceneRendering() has packed the records (processDrawables() does
// the three steps in that order).  Matrices are column-major float[16].
#pragma once

#include <array>
#include <cstddef>
#include <cstdint>
#include <functional>
#include <memory>
#include <vector>

#include "DataStorage.h"
#include "ParentChildList.h"

#if __has_include(<glm/mat4x4.hpp>) && !defined(CADR_FACADE_NO_GLM)
#include <glm/mat4x4.hpp>
#endif

namespace CadR {

// The matrix type of MatrixList: glm::mat4 where GLM is on the include
// path (as in the reference, src/CadR/MatrixList.h:33-36), else 16 floats
// in column-major order.  The library itself only moves 64-byte blocks, so
// code built either way links against the same library.
#if __has_include(<glm/mat4x4.hpp>) && !defined(CADR_FACADE_NO_GLM)
using Mat4 = glm::mat4;
#else
using Mat4 = std::array<float, 16>;
#endif
static_assert(sizeof(Mat4) == 64, "a 4x4 float matrix");

struct PrimitiveSet {
    uint32_t indexCount;
    uint32_t startIndex;
};
static_assert(sizeof(PrimitiveSet) == 8, "PrimitiveSet layout");

struct DrawableGpuData {
    uint64_t vertexDataHandle;
    uint64_t indexDataHandle;
    uint64_t matrixListHandle;
    uint64_t drawableDataHandle;
    uint64_t primitiveSetHandle;
    uint32_t primitiveSetOffset;
    uint32_t padding;

    DrawableGpuData() = default;
    constexpr DrawableGpuData(uint64_t vertexData, uint64_t indexData, uint64_t matrixList, uint64_t drawableData,
                              uint64_t primitiveSet, uint32_t primitiveSetOffset_)
        : vertexDataHandle(vertexData), indexDataHandle(indexData), matrixListHandle(matrixList),
          drawableDataHandle(drawableData), primitiveSetHandle(primitiveSet), primitiveSetOffset(primitiveSetOffset_),
          padding(0)
    {
    }
};
static_assert(sizeof(DrawableGpuData) == 48, "DrawableGpuData must be 48 bytes (Drawable.cpp:13)");
static_assert(sizeof(DrawableGpuData) == sizeof(cadr_drawable_gpu_data), "C ABI record");

class Renderer;
class StateSet;

class Geometry {
public:
    Geometry(Renderer& r);
    Geometry(Geometry&&) = default;
    Geometry(const Geometry&) = delete;
    Geometry& operator=(const Geometry&) = delete;
    Geometry& operator=(Geometry&&) = default;
    Renderer& renderer() const { return *_renderer; }
    DataStorage& dataStorage() const { return _vertices.dataStorage(); }
    size_t vertexDataSize() const { return _vertices.size(); }
    size_t indexDataSize() const { return _indices.size(); }
    size_t primitiveSetDataSize() const { return _primitiveSets.size(); }
    DataAllocation& vertexDataAllocation() { return _vertices; }
    const DataAllocation& vertexDataAllocation() const { return _vertices; }
    DataAllocation& indexDataAllocation() { return _indices; }
    const DataAllocation& indexDataAllocation() const { return _indices; }
    DataAllocation& primitiveSetDataAllocation() { return _primitiveSets; }
    const DataAllocation& primitiveSetDataAllocation() const { return _primitiveSets; }
    void uploadVertexData(const void* p, size_t n) { _vertices.upload(p, n); }
    void uploadIndexData(const void* p, size_t n) { _indices.upload(p, n); }
    void uploadPrimitiveSetData(const void* p, size_t n) { _primitiveSets.upload(p, n); }
    StagingData createVertexStagingData(size_t n) { return _vertices.alloc(n); }
    StagingData createIndexStagingData(size_t n) { return _indices.alloc(n); }
    StagingData createPrimitiveSetStagingData(size_t n) { return _primitiveSets.alloc(n); }
    void freeVertexData() { _vertices.free(); }
    void freeIndexData() { _indices.free(); }
    void freePrimitiveSetData() { _primitiveSets.free(); }
    void freeData()
    {
        freeVertexData();
        freeIndexData();
        freePrimitiveSetData();
    }

private:
    Renderer* _renderer;
    DataAllocation _vertices, _indices, _primitiveSets;
};

class MatrixList {
public:
    MatrixList(Renderer& r);
    MatrixList(MatrixList&&) = default;
    void setMatrices(const Mat4& m) { setMatrixData(&m, 1); }
    void setMatrices(const std::vector<Mat4>& m) { setMatrixData(m.data(), m.size()); }
    void setMatrices(const Mat4* m, size_t n) { setMatrixData(m, n); }
    // A new content of `n` matrices (header written), to be filled in place.
    Mat4* editNewContent(size_t n) { return static_cast<Mat4*>(newContent(n)); }
    uint64_t handle() const { return _list.handle(); }
    uint64_t deviceAddress() const { return _list.deviceAddress(); }

    // The 64-byte header {numMatrices, capacity, 0...} followed by n
    // column-major 64-byte matrices (MatrixList.h:54-59).
    void setMatrixData(const void* matrices, size_t n);
    void* newContent(size_t n);

private:
    DataAllocation _list;
};

class Drawable {
public:
    Drawable() = default;
    Drawable(Geometry& g, uint32_t primitiveSetOffset, MatrixList& ml, StateSet& ss);
    Drawable(Geometry& g, uint32_t primitiveSetOffset, MatrixList& ml, DataAllocation& drawableData, StateSet& ss);
    Drawable(Drawable&& other) noexcept;
    Drawable(const Drawable&) = delete;
    Drawable& operator=(const Drawable&) = delete;
    Drawable& operator=(Drawable&& rhs) noexcept;
    ~Drawable();
    // (Re)creates the drawable in `ss`, leaving the StateSet it was in.
    void create(Geometry& g, uint32_t primitiveSetOffset, MatrixList& ml, StateSet& ss);
    void create(Geometry& g, uint32_t primitiveSetOffset, MatrixList& ml, DataAllocation& drawableData, StateSet& ss);
    void destroy() noexcept;
    bool isValid() const { return _index != ~0u; }
    Renderer& renderer() const;
    // The StateSet that draws it, or drew it last (after destroy()).
    StateSet& stateSet() const { return *_stateSet; }
    MatrixList& matrixList() const { return *_matrixList; }
    DataAllocation* drawableData() const { return _drawableData; }

private:
    void create(Geometry& g, uint32_t primitiveSetOffset, MatrixList& ml, DataAllocation* drawableData, StateSet& ss);
    StateSet* _stateSet = nullptr;
    MatrixList* _matrixList = nullptr;
    DataAllocation* _drawableData = nullptr;
    uint32_t _index = ~0u;
    friend class StateSet;
};

// What StateSet::recordToCommandBuffer records for one StateSet with
// drawables: cmdPushConstants(offset 8, pointersBase + first*32) and
// cmdDrawIndirect(indirectBuffer, first*16, count, 16) (StateSet.cpp:240-258).
struct DrawCall {
    const StateSet* stateSet;
    uint64_t first;              // drawableCounter
    uint32_t count;
    uint64_t drawablePointers;   // device address of the region's DrawablePointers
    uint64_t indirectOffset;     // byte offset into the indirect buffer
};

class StateSet {
public:
    StateSet(Renderer& r) : _renderer(&r) {}
    ~StateSet();
    StateSet(const StateSet&) = delete;
    StateSet& operator=(const StateSet&) = delete;

    Renderer& renderer() const { return *_renderer; }
    bool forceRecording() const { return _forceRecording; }
    // Detaches every drawable (as the destructor does).
    void destroy() noexcept { removeAllDrawables(); }
    // Moves `d` here with record `g` (out of the StateSet it was in).
    void appendDrawable(Drawable& d, const DrawableGpuData& g);
    static void removeDrawable(Drawable& d) noexcept;
    void removeAllDrawables() noexcept;
    Drawable& getDrawable(size_t index) const { return *_drawables[index]; }
    // From a prepareCallList function: record this StateSet in this frame
    // even without drawables.
    void requestRecording() { _skipRecording = false; }
    void appendChild(StateSet& child) { childList.append(child); }
    // Removes the first relation to `child`, if any.
    void removeChild(StateSet& child);
    size_t getNumDrawables() const { return _records.size(); }
    const std::vector<DrawableGpuData>& drawableDataList() const { return _records; }
    void setForceRecording(bool v) { _forceRecording = v; }

    // Called at the start of prepareRecording(), before the children.
    std::vector<std::function<void(StateSet&)>> prepareCallList;

    size_t prepareRecording();
    void recordToCommandBuffer(std::vector<DrawCall>& out, size_t& drawableCounter);
    // The same draw calls without the copy of the records (their packed
    // array is on the device: Renderer::processDrawablesResident).
    void recordDrawCalls(std::vector<DrawCall>& out, size_t& drawableCounter) const;

    // Where childList and parentList lie in a StateSet
    // (src/CadR/StateSet.h:77-79).
    static const ParentChildListOffsets parentChildListOffsets;
    ChildList<StateSet, parentChildListOffsets> childList;
    ParentList<StateSet, parentChildListOffsets> parentList;

private:
    void append(Drawable& d, const DrawableGpuData& g);
    void remove(Drawable& d) noexcept;
    Renderer* _renderer;
    bool _skipRecording = true;
    bool _forceRecording = false;
    std::vector<DrawableGpuData> _records;
    std::vector<Drawable*> _drawables;
    std::vector<uint32_t> _slots;  // the records' slots in the renderer's device-resident pack
    friend class Drawable;
    friend class Renderer;
};

// CadR::FrameInfo (src/CadR/FrameInfo.h:15-31), with the reference's
// fields.  CPU timestamps are nanoseconds of the host's steady clock; GPU
// timestamps are nanoseconds too (gpuTimestampPeriod() = 1e-9 s): the
// frame's first GPU timestamp is the host clock when its first GPU work was
// queued, and the others add the CUDA-event durations to it, so their
// differences are exact GPU durations.  gpuBeginFrame equals cpuBeginFrame.
struct FrameInfo {
    size_t frameNumber = ~size_t(0);
    uint64_t gpuBeginFrame = 0;
    uint64_t cpuBeginFrame = 0;
    uint64_t cpuPrepareRecordingBegin = 0;
    uint64_t cpuPrepareRecordingEnd = 0;
    uint64_t cpuRecordStateSetsBegin = 0;
    uint64_t cpuRecordStateSetsEnd = 0;
    std::vector<uint64_t> cpuUserTimestampList;
    uint64_t cpuEndFrame = 0;
    uint64_t gpuBeginExecution = 0;                             // before the frame's uploads
    uint64_t gpuAfterTransfersAndBeforeDrawableProcessing = 0;  // after them
    uint64_t gpuAfterDrawableProcessingAndBeforeRendering = 0;  // after the processDrawables kernel
    uint64_t gpuEndExecution = 0;                               // at the frame's end (no rendering here)
    static constexpr uint32_t gpuTimestampPoolSize = 4;
};

class Renderer {
public:
    // Renderer on CUDA device 0 (or `device`) with its own cadr_context,
    // created at the first use of the device (so that the host side -
    // StateSets, recording, handles - works on a machine without a GPU).
    // With makeDefault it becomes Renderer::get() (Renderer.cpp:64-73).
    explicit Renderer(bool makeDefault = true);
    explicit Renderer(int device, bool makeDefault = true);
    // Renderer over a caller-provided backend; without a context only the
    // host side (allocation, handles, recording) is available.
    explicit Renderer(MemoryBackend& backend, bool makeDefault = true);
    ~Renderer();
    // The default renderer (Renderer.h:109-110, 220-221).
    static Renderer& get() { return *_defaultRenderer; }
    static void set(Renderer& r) noexcept { _defaultRenderer = &r; }
    Renderer(const Renderer&) = delete;
    Renderer& operator=(const Renderer&) = delete;

    DataStorage& dataStorage() { return *_storage; }
    cadr_context* context() const { return _backend->context(); }
    // Frees this renderer's own device buffers (the packed drawables, the
    // indirect and pointer buffers, the device-resident pack) once the
    // context's work has finished.  Idempotent; the destructor calls it
    // (Renderer.cpp:89-94, 316-376).  As in the reference, the renderer
    // is then only destroyed, not used; its DataStorage memory is freed with it.
    void finalize();
    // Forgets those buffers without freeing them, for a context whose
    // device failed (Renderer.cpp:379-387).
    void leakResources() noexcept;
    // Alignment of the device blocks the renderer allocates (cudaMalloc
    // gives 256 bytes), and an offset rounded up to it
    // (Renderer.h:149-150, 228-229).
    size_t standardBufferAlignment() const { return 256; }
    size_t alignStandardBuffer(size_t offset) const { return (offset + 255) & ~size_t(255); }
    size_t frameNumber() const { return _frame; }

    size_t beginFrame();
    size_t prepareSceneRendering(StateSet& root);
    // Frame timing (Renderer.h:155-163 of the reference).  While on, each
    // frame with drawable processing records the four GPU timestamps of
    // FrameInfo; getFrameInfo() returns the last frame ended by endFrame(),
    // waiting for its GPU timestamps (frameNumber stays ~0 when the frame
    // processed no drawables).  useCalibratedTimestamps has no effect.
    bool collectFrameInfo() const { return _collect; }
    void setCollectFrameInfo(bool on, bool useCalibratedTimestamps = false);
    const FrameInfo& getFrameInfo();
    const FrameInfo& getCurrentFrameInfo() const { return _currentInfo; }
    double cpuTimestampPeriod() const { return 1e-9; }
    float gpuTimestampPeriod() const { return 1e-9f; }
    uint64_t getCpuTimestamp() const;
    void recordSceneRendering(StateSet& root, std::vector<DrawCall>& out);
    void recordDrawableProcessing(size_t numDrawables, cadr_stream stream = nullptr);
    void processDrawables(StateSet& root, std::vector<DrawCall>& out, cadr_stream stream = nullptr);
    // processDrawables() with the records device-resident (cadr_pack_*):
    // instead of StateSet::recordToCommandBuffer's copy of every record into
    // staging and its upload, a frame uploads only the records of drawables
    // created since the previous frame, and lays the pack out again only when
    // StateSet membership or list order changed.  Same draw calls, same
    // indirect and DrawablePointers buffers as processDrawables().
    void processDrawablesResident(StateSet& root, std::vector<DrawCall>& out, cadr_stream stream = nullptr);
    void endFrame();
    size_t executeCopyOperations();

    DrawableGpuData* drawableStagingData() const { return _staging.data(); }
    size_t drawableBufferSize() const { return _capacity * sizeof(DrawableGpuData); }
    uint64_t drawableBufferAddress() const { return _drawables; }
    uint64_t drawIndirectBufferAddress() const { return _indirect; }
    uint64_t drawablePointersBufferAddress() const { return _pointers; }
    static constexpr uint32_t drawablePointersRecordSize = 32;

private:
    void growBuffers(size_t numDrawables);
    uint32_t allocSlot(StateSet* owner, const DrawableGpuData& g);
    void freeSlot(uint32_t slot) noexcept;
    void growPack(uint32_t slots);
    // Device-resident records: slot owner (nullptr = free), the records not
    // yet on the device, whether the layout changed.
    cadr_pack* _pack = nullptr;
    uint32_t _packCapacity = 0;
    std::vector<StateSet*> _slotOwner;
    std::vector<uint32_t> _freeSlots;
    std::vector<uint32_t> _newSlots;
    std::vector<DrawableGpuData> _newRecords;
    std::vector<const StateSet*> _tree;  // the StateSets of the last resident frame, in walk order
    void timestamp(uint32_t index, cadr_stream stream);
    bool _collect = false;
    FrameInfo _currentInfo, _lastInfo;
    uint32_t _gpuStamps = 0;             // timestamps the current frame recorded
    cadr_stream _frameStream = nullptr;  // the stream of the current frame's drawable processing
    size_t _endedFrame = ~size_t(0);     // the frame getFrameInfo() reports
    size_t _lastFrameUploadBytes = 0, _currentFrameUploadBytes = 0;
    bool _endedHasGpu = false;
    uint64_t _endedGpuBase = 0;
    bool _layoutDirty = true;
    friend class StateSet;
    static Renderer* _defaultRenderer;
    std::unique_ptr<MemoryBackend> _ownBackend;
    MemoryBackend* _backend;
    std::unique_ptr<DataStorage> _storage;
    size_t _frame = ~size_t(0);
    size_t _capacity = 0;
    uint64_t _drawables = 0, _indirect = 0, _pointers = 0;
    mutable std::vector<DrawableGpuData> _staging;
};

}  // namespace CadR
