// CPU test of cadr::DeviceGuard against a fake CUDA runtime: the three
// runtime calls the guard makes are defined here, over a simulated current
// device per thread, so the test needs neither a GPU nor libcudart.
#include <cstdio>
#include <cstdlib>

#include "../../cadr_gb300/csrc/device_guard.h"

namespace {
int g_current = 0;        // the calling thread's current device
int g_devices = 4;        // devices the fake runtime reports
int g_set_calls = 0;
bool g_fail_set = false;  // make the next cudaSetDevice fail
}  // namespace

extern "C" cudaError_t cudaGetDevice(int* d)
{
    *d = g_current;
    return cudaSuccess;
}

extern "C" cudaError_t cudaSetDevice(int d)
{
    g_set_calls++;
    if (g_fail_set || d < 0 || d >= g_devices) return cudaErrorInvalidDevice;
    g_current = d;
    return cudaSuccess;
}

extern "C" cudaError_t cudaGetLastError(void) { return cudaSuccess; }

#define CHECK(c)                                                        \
    do {                                                                \
        if (!(c)) {                                                     \
            std::fprintf(stderr, "%s:%d: %s failed\n", __FILE__, __LINE__, #c); \
            std::exit(1);                                               \
        }                                                               \
    } while (0)

// An entry point of the library, reduced to its device handling: it works
// on `device` and returns early on an error.
static int entry(int device, bool early_error, int* seen)
{
    cadr::DeviceGuard dg(device);
    if (dg.error() != cudaSuccess) return 2;
    *seen = g_current;
    if (early_error) return 1;
    return 0;
}

int main()
{
    int seen = -1;
    // The caller works on device 2; the library's context is on device 0.
    g_current = 2;
    CHECK(entry(0, false, &seen) == 0);
    CHECK(seen == 0);
    CHECK(g_current == 2);
    // The error path restores too.
    CHECK(entry(0, true, &seen) == 1);
    CHECK(g_current == 2);
    // Same device: no switch at all.
    g_set_calls = 0;
    CHECK(entry(2, false, &seen) == 0);
    CHECK(seen == 2 && g_current == 2 && g_set_calls == 0);
    // A switch that fails is reported and leaves the device alone.
    g_fail_set = true;
    CHECK(entry(1, false, &seen) == 2);
    CHECK(g_current == 2);
    g_fail_set = false;
    // Nested guards (an entry point calling another) unwind in order.
    {
        cadr::DeviceGuard a(1);
        CHECK(g_current == 1);
        {
            cadr::DeviceGuard b(3);
            CHECK(g_current == 3);
        }
        CHECK(g_current == 1);
    }
    CHECK(g_current == 2);
    std::puts("device guard ok");
    return 0;
}
