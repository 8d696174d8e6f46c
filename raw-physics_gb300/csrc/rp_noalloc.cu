// Static device scratch for the no-allocation contact query (rp_contacts_noalloc).
//
// The query writes its contacts into a file-scope __device__ array instead of a buffer the world
// allocates on first use, so a call makes no device (or host heap) allocation. The array's address
// is looked up once per device, the first time the query runs on it (with that device current); that
// first call therefore does the set-up and should come before any stream capture. Nothing in the
// scratch has to start at zero: the kernel writes the count and every contact it reports. There is
// one scratch per device, so calls on the same device must not overlap (they would race on it). The
// cached address lives as long as the loaded module: a cudaDeviceReset while the library is loaded
// would leave it stale, and is not supported.
#include <cuda_runtime.h>
#include <mutex>
#include "rp_launch.h"

namespace rp {

static __device__ __align__(256) double g_noalloc_contacts[NOALLOC_MAX_CONTACTS * 9];
static __device__ __align__(256) int g_noalloc_count;

namespace {
constexpr int kMaxDevices = 64;
std::once_flag g_once[kMaxDevices];
cudaError_t g_setup_rc[kMaxDevices];
double* g_contacts_ptr[kMaxDevices];
int* g_count_ptr[kMaxDevices];
}  // namespace

// Device addresses of the scratch on `device`, which must be the current device.
cudaError_t noalloc_scratch(int device, double** contacts, int** count) {
    if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
    std::call_once(g_once[device], [device] {
        void* p = nullptr;
        cudaError_t rc = cudaGetSymbolAddress(&p, g_noalloc_contacts);
        if (rc == cudaSuccess) {
            g_contacts_ptr[device] = static_cast<double*>(p);
            rc = cudaGetSymbolAddress(&p, g_noalloc_count);
            if (rc == cudaSuccess) g_count_ptr[device] = static_cast<int*>(p);
        }
        g_setup_rc[device] = rc;
    });
    if (g_setup_rc[device] != cudaSuccess) return g_setup_rc[device];
    *contacts = g_contacts_ptr[device];
    *count = g_count_ptr[device];
    return cudaSuccess;
}

}  // namespace rp
