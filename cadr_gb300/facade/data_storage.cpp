// data_storage.cpp - memory backends, DataMemory (two-block circular
// placement), DataStorage (64 KiB / 2 MiB / 32 MiB block strategy),
// DataAllocation and HandlelessAllocation of the C++ facade.
#include <CadR/DataStorage.h>
#include <CadR/Renderer.h>

#include <algorithm>
#include <cstdlib>
#include <string>

namespace CadR {

// ---------------------------------------------------------------------------
// Backends.

CudaMemoryBackend::~CudaMemoryBackend()
{
    if (_own && _ctx) cadr_context_destroy(_ctx);
}

cadr_context* CudaMemoryBackend::context() const
{
    if (!_ctx && _own) check(cadr_context_create(_device, &_ctx), "Renderer: context");
    return _ctx;
}

uint64_t CudaMemoryBackend::allocBlock(size_t bytes)
{
    void* p = nullptr;
    if (cadr_device_alloc(context(), bytes, &p) != CADR_OK) return 0;
    return reinterpret_cast<uint64_t>(p);
}

void CudaMemoryBackend::freeBlock(uint64_t address) noexcept
{
    if (_ctx) cadr_device_free(_ctx, reinterpret_cast<void*>(address));
}

void CudaMemoryBackend::upload(uint64_t dst, const void* src, size_t bytes)
{
    check(cadr_upload(context(), reinterpret_cast<void*>(dst), src, bytes, nullptr), "DataStorage upload");
}

void CudaMemoryBackend::flush() {}

HostMemoryBackend::HostMemoryBackend(size_t arenaBytes)
{
    _bytes = (arenaBytes + 255) & ~size_t(255);
    _arena = static_cast<uint8_t*>(std::aligned_alloc(256, _bytes));
    if (!_arena) throw OutOfResources("HostMemoryBackend: cannot allocate the arena");
    std::memset(_arena, 0, _bytes);
    _free[0] = _bytes;
}

HostMemoryBackend::~HostMemoryBackend() { std::free(_arena); }

uint64_t HostMemoryBackend::allocBlock(size_t bytes)
{
    bytes = (bytes + 255) & ~size_t(255);
    for (auto it = _free.begin(); it != _free.end(); ++it) {
        if (it->second >= bytes) {
            const uint64_t off = it->first;
            const size_t rest = it->second - bytes;
            _free.erase(it);
            if (rest) _free[off + bytes] = rest;
            _used[off] = bytes;
            return reinterpret_cast<uint64_t>(_arena) + off;
        }
    }
    return 0;
}

void HostMemoryBackend::freeBlock(uint64_t address) noexcept
{
    const uint64_t off = address - reinterpret_cast<uint64_t>(_arena);
    auto u = _used.find(off);
    if (u == _used.end()) return;
    auto it = _free.emplace(off, u->second).first;
    _used.erase(u);
    auto nx = std::next(it);
    if (nx != _free.end() && it->first + it->second == nx->first) {
        it->second += nx->second;
        _free.erase(nx);
    }
    if (it != _free.begin()) {
        auto pv = std::prev(it);
        if (pv->first + pv->second == it->first) {
            pv->second += it->second;
            _free.erase(it);
        }
    }
}

void HostMemoryBackend::upload(uint64_t dst, const void* src, size_t bytes)
{
    std::memcpy(reinterpret_cast<void*>(dst), src, bytes);
}

// ---------------------------------------------------------------------------
// DataMemory.

DataMemory::DataMemory(DataStorage& storage, uint64_t address, size_t size)
    : _storage(&storage), _base(address), _size(size), _end(address + size), _b1Start(address), _b1End(address),
      _b2End(address)
{
}

DataMemory::~DataMemory()
{
    for (auto& kv : _block1) delete kv.second;
    for (auto& kv : _block2) delete kv.second;
}

// CircularAllocationMemory::allocPropose + alloc{1,2}Commit: append to
// block 1 while it fits before the buffer end, else to block 2 (from the
// buffer start up to block 1's start).
DataAllocationRecord* DataMemory::alloc(size_t n)
{
    const uint64_t align = n >= 64 ? 64 : 16;
    int block = 0;
    uint64_t addr = 0, prevEnd = 0;
    if (_b1End + n <= _end) {
        const uint64_t a = (_b1End + align - 1) & ~(align - 1);
        if (a + n <= _end) {
            block = 1;
            addr = a;
            prevEnd = _b1End;
        }
    }
    if (!block && _b2End + n <= _b1Start) {
        const uint64_t a = (_b2End + align - 1) & ~(align - 1);
        if (a + n <= _b1Start) {
            block = 2;
            addr = a;
            prevEnd = _b2End;
        }
    }
    if (!block) return nullptr;
    auto* r = new DataAllocationRecord();
    r->deviceAddress = addr;
    r->size = n;
    r->dataMemory = this;
    r->block = block;
    r->span = addr + n - prevEnd;
    _usedBytes += r->span;
    if (block == 1) {
        _b1End = addr + n;
        _block1[addr] = r;
    } else {
        _b2End = addr + n;
        _block2[addr] = r;
    }
    return r;
}

// Freeing the first allocation of a block moves the block start to the
// next live allocation; an empty block 1 is replaced by block 2 (or reset
// to the buffer start when block 2 is empty too).
void DataMemory::release(DataAllocationRecord* r) noexcept
{
    _usedBytes -= r->span;
    if (r->block == 1) {
        const bool first = !_block1.empty() && _block1.begin()->first == r->deviceAddress;
        _block1.erase(r->deviceAddress);
        if (_block1.empty()) {
            if (!_block2.empty()) {
                _block1.swap(_block2);
                for (auto& kv : _block1) kv.second->block = 1;
                _b1Start = _block1.begin()->first;
                _b1End = _b2End;
                _b2End = _base;
            } else {
                _b1Start = _b1End = _b2End = _base;
            }
        } else if (first) {
            _b1Start = _block1.begin()->first;
        }
    } else {
        _block2.erase(r->deviceAddress);
        if (_block2.empty()) _b2End = _base;
    }
    delete r;
}

void DataMemory::free(DataAllocationRecord* a) noexcept
{
    if (!a || a->size == 0 || !a->dataMemory) return;
    DataStorage& s = *a->dataMemory->_storage;
    if (a->pending) {
        auto it = std::find(s._pending.begin(), s._pending.end(), a);
        if (it != s._pending.end()) {
            *it = s._pending.back();
            s._pending.pop_back();
        }
    }
    a->dataMemory->release(a);
}

// ---------------------------------------------------------------------------
// DataStorage.

DataStorage::DataStorage(MemoryBackend& backend) : _backend(&backend), _handles(*this) {}

DataStorage::~DataStorage()
{
    // The tables live in this storage's memory: free them before it goes.
    _handles.destroyAll();
    _pending.clear();
    for (DataMemory* m : _memories) {
        _backend->freeBlock(m->deviceAddress());
        delete m;
    }
}

DataMemory* DataStorage::createMemory(size_t bytes)
{
    const uint64_t a = _backend->allocBlock(bytes);
    if (!a)
        throw OutOfResources("CadR::DataStorage::alloc() error: Cannot allocate DataMemory. Requested size: " +
                             std::to_string(bytes) + " bytes.");
    auto* m = new DataMemory(*this, a, bytes);
    _memories.push_back(m);
    return m;
}

// DataStorage::allocInternal (src/CadR/DataStorage.cpp:31-96).
DataAllocationRecord* DataStorage::allocInternal(size_t n)
{
    if (!_first)
        _first = createMemory(n < smallMemorySize ? smallMemorySize
                              : n < mediumMemorySize ? mediumMemorySize
                                                     : std::max(n, largeMemorySize));
    DataAllocationRecord* a = _first->alloc(n);
    if (a) return a;
    if (!_second) _second = createMemory(n < mediumMemorySize ? mediumMemorySize : std::max(n, largeMemorySize));
    a = _second->alloc(n);
    if (a) return a;
    DataMemory* m = createMemory(std::max(largeMemorySize, n));
    _first = _second;
    _second = m;
    a = _second->alloc(n);
    if (!a) throw OutOfResources("CadR::DataStorage::alloc() error: Cannot allocate DataAllocation.");
    return a;
}

DataAllocationRecord* DataStorage::alloc(size_t n)
{
    if (n == 0) return &_zero;
    DataAllocationRecord* a = allocInternal(n);
    a->stagingFrameNumber = _frame;
    return a;
}

DataAllocationRecord* DataStorage::realloc(DataAllocationRecord* old, size_t n)
{
    if (n == 0) {
        free(old);
        return &_zero;
    }
    DataAllocationRecord* a = allocInternal(n);
    a->stagingFrameNumber = _frame;
    if (old->size != 0) DataMemory::free(old);
    return a;
}

void DataStorage::free(DataAllocationRecord* a) noexcept
{
    if (a->size == 0) return;
    DataMemory::free(a);
}

void DataStorage::markPending(DataAllocationRecord* a)
{
    if (a->size == 0 || a->pending) return;
    a->pending = true;
    _pending.push_back(a);
}

// Uploads all staged content.  Pending allocations of one DataMemory that
// lie within 256 bytes of each other go up as one copy; the gaps between
// them belong to no live allocation and are written with zeros.
size_t DataStorage::uploadPending()
{
    size_t bytes = 0;
    std::sort(_pending.begin(), _pending.end(),
              [](const DataAllocationRecord* x, const DataAllocationRecord* y) { return x->deviceAddress < y->deviceAddress; });
    std::vector<uint8_t> run;
    size_t i = 0;
    while (i < _pending.size()) {
        DataAllocationRecord* r0 = _pending[i];
        uint64_t start = r0->deviceAddress, end = start + r0->size;
        size_t j = i + 1;
        while (j < _pending.size() && _pending[j]->dataMemory == r0->dataMemory &&
               _pending[j]->deviceAddress <= end + 256) {
            end = std::max<uint64_t>(end, _pending[j]->deviceAddress + _pending[j]->size);
            j++;
        }
        if (j == i + 1) {
            _backend->upload(start, r0->staging.data(), r0->size);
        } else {
            run.assign(end - start, 0);
            for (size_t k = i; k < j; k++)
                std::memcpy(run.data() + (_pending[k]->deviceAddress - start), _pending[k]->staging.data(),
                            _pending[k]->size);
            _backend->upload(start, run.data(), run.size());
        }
        bytes += end - start;
        for (size_t k = i; k < j; k++) {
            _pending[k]->pending = false;
            std::vector<uint8_t>().swap(_pending[k]->staging);
        }
        i = j;
    }
    _pending.clear();
    _handles.uploadDirty();
    _backend->flush();
    return bytes;
}

// ---------------------------------------------------------------------------
// DataAllocation / HandlelessAllocation (DataAllocation.cpp:18-70).

namespace {
// The record of an allocation bound to no storage (DataAllocation(nullptr)).
DataAllocationRecord g_nullRecord;
DataAllocationRecord* emptyRecord(DataStorage* s) { return s ? s->zeroSizeAllocationRecord() : &g_nullRecord; }
}  // namespace

DataAllocation::DataAllocation(std::nullptr_t) noexcept : _storage(nullptr), _record(&g_nullRecord), _handle(0) {}

DataAllocation::DataAllocation(DataStorage& storage)
    : _storage(&storage), _record(storage.zeroSizeAllocationRecord()), _handle(storage.createHandle())
{
}

DataAllocation::DataAllocation(DataStorage& storage, noHandle_t) noexcept
    : _storage(&storage), _record(storage.zeroSizeAllocationRecord()), _handle(0)
{
}

DataAllocation::DataAllocation(Renderer& r) : DataAllocation(r.dataStorage()) {}

DataAllocation::DataAllocation(Renderer& r, noHandle_t) noexcept : DataAllocation(r.dataStorage(), noHandle) {}

DataAllocation::DataAllocation(DataAllocation&& o) noexcept : _storage(o._storage), _record(o._record), _handle(o._handle)
{
    o._record = emptyRecord(_storage);
    o._handle = 0;
}

void DataAllocation::init(DataStorage& storage)
{
    free();
    if (_handle && _storage != &storage) {
        _storage->destroyHandle(_handle);
        _handle = storage.createHandle();
    }
    _storage = &storage;
    _record = storage.zeroSizeAllocationRecord();
}

StagingData DataAllocation::alloc()
{
    if (_record->size != 0 && _record->stagingFrameNumber == _storage->frameNumber()) return StagingData(_record, false);
    return alloc(_record->size);
}

uint64_t DataAllocation::createHandle(DataStorage& storage)
{
    if (_handle == 0) {
        _storage = &storage;
        _handle = storage.createHandle();
        if (_record->size) storage.setHandle(_handle, _record->deviceAddress);
    }
    return _handle;
}

void DataAllocation::destroyHandle() noexcept
{
    if (_handle == 0) return;
    _storage->destroyHandle(_handle);
    _handle = 0;
}

size_t DataAllocation::offset() const { return size_t(_record->deviceAddress - _record->dataMemory->deviceAddress()); }

DataAllocation& DataAllocation::operator=(DataAllocation&& o) noexcept
{
    if (this == &o) return *this;
    free();
    if (_handle) _storage->destroyHandle(_handle);
    _storage = o._storage;
    _record = o._record;
    _handle = o._handle;
    o._record = emptyRecord(_storage);
    o._handle = 0;
    return *this;
}

DataAllocation::~DataAllocation()
{
    if (!_storage) return;
    free();
    if (_handle) _storage->destroyHandle(_handle);
}

StagingData DataAllocation::alloc(size_t n)
{
    const bool reuse = _record->size != 0 && _record->stagingFrameNumber == _storage->frameNumber() && n <= _record->size;
    if (reuse) {
        _record->size = n;
    } else {
        _record = _storage->realloc(_record, n);
        if (_handle) _storage->setHandle(_handle, _record->deviceAddress);
    }
    _record->staging.resize(_record->size);
    _storage->markPending(_record);
    return StagingData(_record, !reuse);
}

void DataAllocation::free() noexcept
{
    if (_record->size == 0) return;
    _storage->free(_record);
    _record = _storage->zeroSizeAllocationRecord();
}

void DataAllocation::upload(const void* p, size_t n)
{
    StagingData s = alloc(n);
    if (n) std::memcpy(s.data(), p, n);
}

HandlelessAllocation::HandlelessAllocation(std::nullptr_t) noexcept : _storage(nullptr), _record(&g_nullRecord) {}

HandlelessAllocation::HandlelessAllocation(DataStorage& storage)
    : _storage(&storage), _record(storage.zeroSizeAllocationRecord())
{
}

HandlelessAllocation::HandlelessAllocation(Renderer& r) : HandlelessAllocation(r.dataStorage()) {}

HandlelessAllocation::HandlelessAllocation(HandlelessAllocation&& o) noexcept : _storage(o._storage), _record(o._record)
{
    o._record = emptyRecord(_storage);
}

HandlelessAllocation& HandlelessAllocation::operator=(HandlelessAllocation&& o) noexcept
{
    if (this == &o) return *this;
    free();
    _storage = o._storage;
    _record = o._record;
    o._record = emptyRecord(_storage);
    return *this;
}

HandlelessAllocation::~HandlelessAllocation()
{
    if (_storage) free();
}

void HandlelessAllocation::init(DataStorage& storage)
{
    free();
    _storage = &storage;
    _record = storage.zeroSizeAllocationRecord();
}

StagingData HandlelessAllocation::alloc()
{
    if (_record->size != 0 && _record->stagingFrameNumber == _storage->frameNumber()) return StagingData(_record, false);
    return alloc(_record->size);
}

StagingData HandlelessAllocation::alloc(size_t n)
{
    const bool reuse = _record->size != 0 && _record->stagingFrameNumber == _storage->frameNumber() && n <= _record->size;
    if (reuse)
        _record->size = n;
    else
        _record = _storage->realloc(_record, n);
    _record->staging.resize(_record->size);
    _storage->markPending(_record);
    return StagingData(_record, !reuse);
}

void HandlelessAllocation::free() noexcept
{
    if (_record->size == 0) return;
    _storage->free(_record);
    _record = _storage->zeroSizeAllocationRecord();
}

}  // namespace CadR
