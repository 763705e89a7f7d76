// export.cu - output buffers a Vulkan renderer can import without a copy.
//
// The reference shares memory between APIs by allocating it exportable and
// handing an opaque POSIX file descriptor to the importer, which takes
// ownership of the descriptor (examples/OpenGLInteroperability/main.cpp:
// 1488-1490 allocates with eOpaqueFd, 1538-1550 gets the FDs, 1616-1619
// imports them).  Here the exporter is CUDA: the buffer is physical device
// memory made with cuMemCreate for POSIX-FD export, mapped into this
// context's address space; cuMemExportToShareableHandle gives the FD that
// Vulkan imports as VK_EXTERNAL_MEMORY_HANDLE_TYPE_OPAQUE_FD_BIT
// (VkImportMemoryFdInfoKHR), and that cuMemImportFromShareableHandle maps
// back into a CUDA context.  Driver entry points are reached through the
// runtime, so the library needs no link against the driver library.
#include <cudaTypedefs.h>

#include "capi_internal.h"

struct cadr_shared_buffer {
    cadr_context* ctx = nullptr;
    CUmemGenericAllocationHandle handle = 0;
    CUdeviceptr ptr = 0;
    size_t bytes = 0;      // mapped size (a multiple of the allocation granularity)
    bool mapped = false;
};

namespace cadr {

namespace {

struct Vmm {
    PFN_cuDeviceGetAttribute_v2000 get_attribute = nullptr;
    PFN_cuMemGetAllocationGranularity_v10020 granularity = nullptr;
    PFN_cuMemCreate_v10020 create = nullptr;
    PFN_cuMemRelease_v10020 release = nullptr;
    PFN_cuMemAddressReserve_v10020 reserve = nullptr;
    PFN_cuMemAddressFree_v10020 address_free = nullptr;
    PFN_cuMemMap_v10020 map = nullptr;
    PFN_cuMemUnmap_v10020 unmap = nullptr;
    PFN_cuMemSetAccess_v10020 set_access = nullptr;
    PFN_cuMemExportToShareableHandle_v10020 export_handle = nullptr;
    PFN_cuMemImportFromShareableHandle_v10020 import_handle = nullptr;
    bool ok = false;
};

template <typename F>
bool entry(const char* name, unsigned version, F& fn)
{
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion(name, &p, version, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
        return false;
    fn = reinterpret_cast<F>(p);
    return true;
}

const Vmm& vmm()
{
    static const Vmm v = [] {
        Vmm t;
        t.ok = entry("cuDeviceGetAttribute", 2000, t.get_attribute) &&
               entry("cuMemGetAllocationGranularity", 10020, t.granularity) &&
               entry("cuMemCreate", 10020, t.create) && entry("cuMemRelease", 10020, t.release) &&
               entry("cuMemAddressReserve", 10020, t.reserve) &&
               entry("cuMemAddressFree", 10020, t.address_free) && entry("cuMemMap", 10020, t.map) &&
               entry("cuMemUnmap", 10020, t.unmap) && entry("cuMemSetAccess", 10020, t.set_access) &&
               entry("cuMemExportToShareableHandle", 10020, t.export_handle) &&
               entry("cuMemImportFromShareableHandle", 10020, t.import_handle);
        return t;
    }();
    return v;
}

cadr_status driver_fail(CUresult r, const char* what)
{
    return fail(CADR_ERR_CUDA, "%s: driver error %d", what, (int)r);
}

CUmemAllocationProp fd_prop(int device)
{
    CUmemAllocationProp p = {};
    p.type = CU_MEM_ALLOCATION_TYPE_PINNED;
    p.location.type = CU_MEM_LOCATION_TYPE_DEVICE;
    p.location.id = device;
    p.requestedHandleTypes = CU_MEM_HANDLE_TYPE_POSIX_FILE_DESCRIPTOR;
    return p;
}

// Device, VMM and POSIX-FD export support, and the allocation granularity.
cadr_status check_support(cadr_context* ctx, size_t* gran)
{
    const Vmm& v = vmm();
    if (!v.ok) return fail(CADR_ERR_CUDA, "shared buffer: driver entry points unavailable");
    int vmm_ok = 0, fd_ok = 0;
    CUresult r = v.get_attribute(&vmm_ok, CU_DEVICE_ATTRIBUTE_VIRTUAL_MEMORY_MANAGEMENT_SUPPORTED, ctx->device);
    if (r == CUDA_SUCCESS)
        r = v.get_attribute(&fd_ok, CU_DEVICE_ATTRIBUTE_HANDLE_TYPE_POSIX_FILE_DESCRIPTOR_SUPPORTED, ctx->device);
    if (r != CUDA_SUCCESS) return driver_fail(r, "shared buffer: device attributes");
    if (!vmm_ok || !fd_ok) return fail(CADR_ERR_CUDA, "shared buffer: the device cannot export POSIX file descriptors");
    const CUmemAllocationProp p = fd_prop(ctx->device);
    r = v.granularity(gran, &p, CU_MEM_ALLOC_GRANULARITY_MINIMUM);
    if (r != CUDA_SUCCESS) return driver_fail(r, "shared buffer: granularity");
    return CADR_OK;
}

// Maps `b->handle` (b->bytes) read-write for the context's device.
cadr_status map_handle(cadr_shared_buffer* b)
{
    const Vmm& v = vmm();
    CUresult r = v.reserve(&b->ptr, b->bytes, 0, 0, 0);
    if (r != CUDA_SUCCESS) return driver_fail(r, "shared buffer: reserve address range");
    r = v.map(b->ptr, b->bytes, 0, b->handle, 0);
    if (r != CUDA_SUCCESS) {
        v.address_free(b->ptr, b->bytes);
        b->ptr = 0;
        return driver_fail(r, "shared buffer: map");
    }
    CUmemAccessDesc a = {};
    a.location.type = CU_MEM_LOCATION_TYPE_DEVICE;
    a.location.id = b->ctx->device;
    a.flags = CU_MEM_ACCESS_FLAGS_PROT_READWRITE;
    r = v.set_access(b->ptr, b->bytes, &a, 1);
    if (r != CUDA_SUCCESS) {
        v.unmap(b->ptr, b->bytes);
        v.address_free(b->ptr, b->bytes);
        b->ptr = 0;
        return driver_fail(r, "shared buffer: set access");
    }
    b->mapped = true;
    return CADR_OK;
}

void release(cadr_shared_buffer* b)
{
    const Vmm& v = vmm();
    if (b->mapped) {
        v.unmap(b->ptr, b->bytes);
        v.address_free(b->ptr, b->bytes);
    }
    if (b->handle) v.release(b->handle);
    delete b;
}

}  // namespace

}  // namespace cadr

using namespace cadr;

extern "C" {

CADR_API cadr_status cadr_shared_buffer_create(cadr_context* ctx, size_t bytes, cadr_shared_buffer** out)
{
    if (!ctx || !out || bytes == 0) return fail(CADR_ERR_INVALID_ARG, "shared_buffer_create: bad argument");
    DeviceGuard dg(ctx->device);
    *out = nullptr;
    size_t gran = 0;
    cadr_status st = check_support(ctx, &gran);
    if (st != CADR_OK) return st;
    auto* b = new cadr_shared_buffer();
    b->ctx = ctx;
    b->bytes = (bytes + gran - 1) / gran * gran;
    const CUmemAllocationProp p = fd_prop(ctx->device);
    const CUresult r = vmm().create(&b->handle, b->bytes, &p, 0);
    if (r != CUDA_SUCCESS) {
        b->handle = 0;
        release(b);
        return r == CUDA_ERROR_OUT_OF_MEMORY ? fail(CADR_ERR_OUT_OF_MEMORY, "shared_buffer_create: device memory")
                                             : driver_fail(r, "shared_buffer_create");
    }
    st = map_handle(b);
    if (st != CADR_OK) {
        release(b);
        return st;
    }
    *out = b;
    return CADR_OK;
}

CADR_API cadr_status cadr_shared_buffer_import_fd(cadr_context* ctx, int fd, size_t bytes, cadr_shared_buffer** out)
{
    if (!ctx || !out || fd < 0 || bytes == 0) return fail(CADR_ERR_INVALID_ARG, "shared_buffer_import_fd: bad argument");
    DeviceGuard dg(ctx->device);
    *out = nullptr;
    size_t gran = 0;
    cadr_status st = check_support(ctx, &gran);
    if (st != CADR_OK) return st;
    if (bytes % gran) return fail(CADR_ERR_INVALID_ARG, "shared_buffer_import_fd: size is not the exported size");
    auto* b = new cadr_shared_buffer();
    b->ctx = ctx;
    b->bytes = bytes;
    const CUresult r = vmm().import_handle(&b->handle, reinterpret_cast<void*>(static_cast<intptr_t>(fd)),
                                           CU_MEM_HANDLE_TYPE_POSIX_FILE_DESCRIPTOR);
    if (r != CUDA_SUCCESS) {
        b->handle = 0;
        release(b);
        return driver_fail(r, "shared_buffer_import_fd");
    }
    st = map_handle(b);
    if (st != CADR_OK) {
        release(b);
        return st;
    }
    // The import holds the allocation; the descriptor is the caller's to close.
    *out = b;
    return CADR_OK;
}

CADR_API cadr_status cadr_shared_buffer_export_fd(cadr_shared_buffer* b, int* fd)
{
    if (!b || !fd) return fail(CADR_ERR_INVALID_ARG, "shared_buffer_export_fd: null argument");
    *fd = -1;
    int f = -1;
    const CUresult r = vmm().export_handle(&f, b->handle, CU_MEM_HANDLE_TYPE_POSIX_FILE_DESCRIPTOR, 0);
    if (r != CUDA_SUCCESS) return driver_fail(r, "shared_buffer_export_fd");
    *fd = f;
    return CADR_OK;
}

CADR_API void* cadr_shared_buffer_device_ptr(cadr_shared_buffer* b)
{
    return b ? reinterpret_cast<void*>(static_cast<uintptr_t>(b->ptr)) : nullptr;
}

CADR_API size_t cadr_shared_buffer_size(cadr_shared_buffer* b) { return b ? b->bytes : 0; }

CADR_API cadr_status cadr_shared_buffer_destroy(cadr_shared_buffer* b)
{
    if (!b) return CADR_OK;
    DeviceGuard dg(b->ctx->device);
    // Work on the buffer may still be queued: it finishes before the
    // mapping goes.
    const cudaError_t e = cudaDeviceSynchronize();
    release(b);
    return e == cudaSuccess ? CADR_OK : cuda_fail(e, "shared_buffer_destroy: synchronize");
}

}  // extern "C"
