// CadR/DataStorage.h - device memory pools, allocations and handles of the
// C++ facade, with the reference's placement and handle rules:
//   * DataStorage sub-allocates DataMemory blocks of 64 KiB, 2 MiB, then
//     32 MiB (src/CadR/DataStorage.cpp:31-96, Renderer.h:104-106);
//   * each DataMemory is a two-block circular allocator: allocations append
//     to block 1, and wrap to block 2 at the buffer start once block 1
//     reaches the end; 16-byte alignment below 64 bytes, 64-byte alignment
//     from 64 bytes on (src/CadR/CircularAllocationMemory.h:521-568);
//   * zero-size allocations share one record at device address 0;
//   * HandleTable hands out 64-bit handles from 1 and resolves them through
//     1, 2 or 3 levels of 2,048-entry tables (src/CadR/HandleTable.cpp).
// Device memory comes from a MemoryBackend: CudaMemoryBackend (device
// memory of a cadr_context, uploads through cadr_upload) or
// HostMemoryBackend (host memory standing in for the device, for tests).
#pragma once

#include <array>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <vector>

#include "Exceptions.h"

namespace CadR {

class DataMemory;
class DataStorage;
class Renderer;

// Where device memory blocks come from and how bytes get there.
class MemoryBackend {
public:
    virtual ~MemoryBackend() = default;
    virtual uint64_t allocBlock(size_t bytes) = 0;        // 256-byte aligned device address, 0 on failure
    virtual void freeBlock(uint64_t address) noexcept = 0;
    virtual void upload(uint64_t dst, const void* src, size_t bytes) = 0;
    virtual void flush() {}                               // order uploads before the next pass
    virtual cadr_context* context() const { return nullptr; }
    // The context if one exists already, without creating it.
    virtual cadr_context* existingContext() const { return context(); }
};

// Device memory of a cadr_context; uploads staged through the context's
// pinned ring on its upload stream.  Either over the caller's context, or
// over one of its own on CUDA device `device`, created at the first use
// and destroyed with the backend.
class CudaMemoryBackend : public MemoryBackend {
public:
    explicit CudaMemoryBackend(cadr_context* ctx) : _ctx(ctx) {}
    explicit CudaMemoryBackend(int device) : _device(device), _own(true) {}
    ~CudaMemoryBackend() override;
    CudaMemoryBackend(const CudaMemoryBackend&) = delete;
    CudaMemoryBackend& operator=(const CudaMemoryBackend&) = delete;
    uint64_t allocBlock(size_t bytes) override;
    void freeBlock(uint64_t address) noexcept override;
    void upload(uint64_t dst, const void* src, size_t bytes) override;
    void flush() override;
    cadr_context* context() const override;
    cadr_context* existingContext() const override { return _ctx; }

private:
    mutable cadr_context* _ctx = nullptr;
    int _device = 0;
    bool _own = false;
};

// Host memory standing in for device memory: one arena whose host addresses
// are the "device" addresses, so host code (the oracle) can follow every
// pointer.
class HostMemoryBackend : public MemoryBackend {
public:
    explicit HostMemoryBackend(size_t arenaBytes = size_t(256) << 20);
    ~HostMemoryBackend() override;
    uint64_t allocBlock(size_t bytes) override;
    void freeBlock(uint64_t address) noexcept override;
    void upload(uint64_t dst, const void* src, size_t bytes) override;
    uint8_t* arena() const { return _arena; }
    size_t arenaBytes() const { return _bytes; }
    size_t usedBlocks() const { return _used.size(); }

private:
    uint8_t* _arena;
    size_t _bytes;
    std::map<uint64_t, size_t> _free;  // offset -> bytes
    std::map<uint64_t, size_t> _used;
};

struct DataAllocationRecord {
    uint64_t deviceAddress = 0;
    size_t size = 0;
    DataMemory* dataMemory = nullptr;
    DataAllocationRecord** recordPointer = nullptr;
    size_t stagingFrameNumber = size_t(-2);
    // facade bookkeeping
    int block = 0;              // 1 or 2: which circular block holds it
    uint64_t span = 0;          // bytes charged to usedBytes (gap before + size)
    std::vector<uint8_t> staging;  // content waiting for the next executeCopyOperations
    bool pending = false;
};

// One device memory block with the two-block circular placement.
class DataMemory {
public:
    DataMemory(DataStorage& storage, uint64_t address, size_t size);
    ~DataMemory();
    DataMemory(const DataMemory&) = delete;
    DataMemory& operator=(const DataMemory&) = delete;

    DataAllocationRecord* alloc(size_t numBytes);   // nullptr when it does not fit
    static void free(DataAllocationRecord* a) noexcept;

    uint64_t deviceAddress() const { return _base; }
    size_t size() const { return _size; }
    size_t usedBytes() const { return _usedBytes; }
    bool empty() const { return _block1.empty() && _block2.empty(); }
    DataStorage& dataStorage() const { return *_storage; }
    // block layout, for white-box tests
    uint64_t block1Start() const { return _b1Start; }
    uint64_t block1End() const { return _b1End; }
    uint64_t block2End() const { return _b2End; }

private:
    void release(DataAllocationRecord* a) noexcept;
    DataStorage* _storage;
    uint64_t _base, _size, _end;
    uint64_t _b1Start, _b1End, _b2End;  // block 2 starts at _base
    size_t _usedBytes = 0;
    std::map<uint64_t, DataAllocationRecord*> _block1, _block2;
};

// Handles -> device addresses, in 1-3 levels of 2,048-entry tables that
// live in the DataStorage themselves (HandleTable.h:33-37).
class HandleTable {
public:
    static constexpr unsigned numHandlesPerTable = 2048;
    static constexpr unsigned handleBitsLevelShift = 11;
    static constexpr unsigned handleBitsLevelMask = 0x07ff;

    explicit HandleTable(DataStorage& storage) : _storage(&storage) {}
    ~HandleTable();
    uint64_t create();
    void set(uint64_t handle, uint64_t addr);
    void destroy(uint64_t handle) noexcept { (void)handle; }  // handles are not recycled, as in the reference
    void destroyAll() noexcept;
    unsigned handleLevel() const { return _level; }
    uint64_t rootTableDeviceAddress() const;
    uint64_t highestHandle() const { return _highest; }
    void uploadDirty();

private:
    struct Table {
        DataAllocationRecord* record = nullptr;  // 16 KiB device copy
        std::array<uint64_t, numHandlesPerTable> addr{};
        bool dirty = true;
    };
    Table* newTable();
    void setEntry(Table* t, unsigned index, uint64_t value);
    DataStorage* _storage;
    std::vector<std::unique_ptr<Table>> _tables;  // every table, for upload and release
    Table* _root = nullptr;
    // level-2 routing table entries and level-3 routing tables
    std::vector<Table*> _llt;      // last-level tables by handle >> 11
    std::vector<Table*> _l1;       // level-1 routing tables (level 3) by handle >> 22
    unsigned _level = 0;
    uint64_t _highest = 0;
};

class DataStorage {
public:
    static constexpr size_t smallMemorySize = 64 << 10;
    static constexpr size_t mediumMemorySize = 2 << 20;
    static constexpr size_t largeMemorySize = 32 << 20;

    explicit DataStorage(MemoryBackend& backend);
    ~DataStorage();
    DataStorage(const DataStorage&) = delete;
    DataStorage& operator=(const DataStorage&) = delete;

    DataAllocationRecord* alloc(size_t numBytes);
    DataAllocationRecord* realloc(DataAllocationRecord* a, size_t numBytes);
    void free(DataAllocationRecord* a) noexcept;
    DataAllocationRecord* zeroSizeAllocationRecord() { return &_zero; }
    std::vector<DataMemory*>& dataMemoryList() { return _memories; }
    const std::vector<DataMemory*>& dataMemoryList() const { return _memories; }
    // The renderer that owns this storage (DataStorage.h: renderer()); null
    // for a storage made directly over a backend.
    Renderer* renderer() const { return _renderer; }
    void setRenderer(Renderer* r) noexcept { _renderer = r; }
    // The bytes staged in the previous frame, which the reference uses to
    // size its staging memory (Renderer.cpp:394-397); kept for callers that
    // read it back.  Staged content here lives in per-allocation host
    // buffers, so nothing else depends on it.
    size_t stagingDataSizeHint() const { return _stagingHint; }
    void setStagingDataSizeHint(size_t bytes) { _stagingHint = bytes; }

    // handles
    uint64_t createHandle() { return _handles.create(); }
    void destroyHandle(uint64_t h) noexcept { _handles.destroy(h); }
    void setHandle(uint64_t h, uint64_t addr) { _handles.set(h, addr); }
    unsigned handleLevel() const { return _handles.handleLevel(); }
    uint64_t handleTableDeviceAddress() const { return _handles.rootTableDeviceAddress(); }
    HandleTable& handleTable() { return _handles; }

    // staged content
    void markPending(DataAllocationRecord* a);
    size_t uploadPending();     // uploads staged content and dirty tables; returns bytes
    MemoryBackend& backend() const { return *_backend; }
    size_t frameNumber() const { return _frame; }
    void setFrameNumber(size_t f) { _frame = f; }

private:
    DataAllocationRecord* allocInternal(size_t numBytes);
    DataMemory* createMemory(size_t bytes);
    MemoryBackend* _backend;
    std::vector<DataMemory*> _memories;
    DataMemory* _first = nullptr;
    DataMemory* _second = nullptr;
    DataAllocationRecord _zero;
    std::vector<DataAllocationRecord*> _pending;
    size_t _frame = ~size_t(0);
    Renderer* _renderer = nullptr;
    size_t _stagingHint = 0;
    HandleTable _handles;
    friend class DataMemory;
};

// Host view of an allocation's new content; uploaded by
// Renderer::executeCopyOperations (StagingData.h in the reference).
class StagingData {
public:
    StagingData() = default;
    // wasReallocated: the allocation moved to new memory for this content,
    // so all of it is to be written (StagingData.h: wasReallocated()).
    explicit StagingData(DataAllocationRecord* r, bool wasReallocated = true) : _r(r), _realloc(wasReallocated) {}
    void* data() const { return _r->staging.data(); }
    template <typename T> T* data() const { return reinterpret_cast<T*>(_r->staging.data()); }
    size_t size() const { return _r->size; }
    size_t sizeInBytes() const { return _r->size; }
    bool wasReallocated() const { return _realloc; }

private:
    DataAllocationRecord* _r = nullptr;
    bool _realloc = false;
};

// An allocation with a handle (DataAllocation.h:45-96).
class DataAllocation {
public:
    enum class noHandle_t : int;
    static constexpr noHandle_t noHandle = noHandle_t(0);
    // An allocation of no storage and no handle, to be init()-ed later.
    // The constructors are implicit, as the reference's are.
    DataAllocation(std::nullptr_t) noexcept;
    DataAllocation(DataStorage& storage);
    DataAllocation(DataStorage& storage, noHandle_t) noexcept;  // without a handle
    DataAllocation(Renderer& r);
    DataAllocation(Renderer& r, noHandle_t) noexcept;
    DataAllocation(DataAllocation&& other) noexcept;
    // Frees this allocation and its handle, then takes other's; other is
    // left empty, without a handle (DataAllocation.h:64, 173).
    DataAllocation& operator=(DataAllocation&& other) noexcept;
    DataAllocation(const DataAllocation&) = delete;
    ~DataAllocation();

    // Frees the memory (the handle stays) and binds to `storage`.
    void init(DataStorage& storage);
    // New content of numBytes; reuses this frame's staging when it fits
    // (DataAllocation.cpp:18-34).
    StagingData alloc(size_t numBytes);
    // New content of the current size; this frame's staging if there is
    // one already (DataAllocation.cpp:37-51).
    StagingData alloc();
    StagingData createStagingData() { return alloc(); }
    StagingData createStagingData(size_t numBytes) { return alloc(numBytes); }
    void free() noexcept;
    // A handle for an allocation made without one, pointed at its current
    // memory (the reference's leaves the entry unset until the next
    // alloc); returns the handle.
    uint64_t createHandle(DataStorage& storage);
    void destroyHandle() noexcept;
    void upload(const void* ptr, size_t numBytes);
    void setData(const void* ptr, size_t numBytes) { upload(ptr, numBytes); }
    template <typename T> void setData(const T& data) { upload(&data, sizeof(data)); }
    template <typename T> T& editNewContent() { return *alloc(sizeof(T)).template data<T>(); }
    template <typename T> T* editNewContent(size_t count) { return alloc(sizeof(T) * count).template data<T>(); }
    uint64_t handle() const { return _handle; }
    uint64_t deviceAddress() const { return _record->deviceAddress; }
    size_t size() const { return _record->size; }
    // The DataMemory block holding a non-empty allocation, and the
    // allocation's offset inside it.
    DataMemory& dataMemory() const { return *_record->dataMemory; }
    size_t offset() const;
    DataStorage& dataStorage() const { return *_storage; }
    Renderer& renderer() const { return *_storage->renderer(); }

private:
    DataStorage* _storage;
    DataAllocationRecord* _record;
    uint64_t _handle;
};

// An allocation without a handle.
class HandlelessAllocation {
public:
    HandlelessAllocation(std::nullptr_t) noexcept;
    HandlelessAllocation(DataStorage& storage);
    HandlelessAllocation(Renderer& r);
    HandlelessAllocation(HandlelessAllocation&& other) noexcept;
    HandlelessAllocation& operator=(HandlelessAllocation&& other) noexcept;
    HandlelessAllocation(const HandlelessAllocation&) = delete;
    ~HandlelessAllocation();

    void init(DataStorage& storage);
    StagingData alloc(size_t numBytes);
    StagingData alloc();
    StagingData createStagingData() { return alloc(); }
    StagingData createStagingData(size_t numBytes) { return alloc(numBytes); }
    void free() noexcept;
    void setData(const void* ptr, size_t numBytes)
    {
        StagingData s = alloc(numBytes);
        if (numBytes) std::memcpy(s.data(), ptr, numBytes);
    }
    template <typename T> void setData(const T& data) { setData(&data, sizeof(data)); }
    template <typename T> T& editNewContent() { return *alloc(sizeof(T)).template data<T>(); }
    template <typename T> T* editNewContent(size_t count) { return alloc(sizeof(T) * count).template data<T>(); }
    uint64_t deviceAddress() const { return _record->deviceAddress; }
    size_t size() const { return _record->size; }
    DataMemory& dataMemory() const { return *_record->dataMemory; }
    size_t offset() const { return size_t(_record->deviceAddress - _record->dataMemory->deviceAddress()); }
    DataStorage& dataStorage() const { return *_storage; }
    Renderer& renderer() const { return *_storage->renderer(); }

private:
    DataStorage* _storage;
    DataAllocationRecord* _record;
};

}  // namespace CadR
