// noalloc.cu -- a tile TSMQR entry point that allocates no device memory.
//
// Who needs it: code that runs inside a host application which owns every byte of device
// memory (its own pool or caching allocator, a fixed memory budget) and therefore may not
// call cudaMalloc itself, and code on latency-critical paths that must not pay for
// cudaMalloc/cudaFree, which can synchronize the whole device and stall other streams.
// palial_gpu_tile_dtsmqr() allocates (and caches) its scratch with cudaMalloc on first use;
// this variant runs the same kernel with its scratch in a fixed array compiled into the
// library instead.
//
// The array holds the two NB x 64 strips the TSMQR kernel works in, for NB up to 512:
// 2 * 512 * 64 doubles = 512 KiB, plus one 256-byte status block.  Every GPU that loads this
// library keeps these 512.25 KiB until the process exits.
#include <cuda_runtime.h>

#include <atomic>
#include <mutex>

#include "../../include/palial_gpu.h"
#include "common.cuh"

namespace palial {
cudaError_t sched_configure();
cudaError_t tile_task_launch(int type, int nb, int ld, double *p0, double *p1, double *p2, double *p3, double *scratch,
                             int *status, cudaStream_t s);
void noalloc_reset();
}  // namespace palial

namespace {
constexpr int kMaxNb = 512;                                   // largest tile size accepted
constexpr size_t kStripDoubles = 2 * (size_t)kMaxNb * 64;    // W and W2 strips
constexpr size_t kStatusDoubles = 32;                         // 256 bytes for the status ints
constexpr int kMaxDevices = 64;

// The scratch itself.  In host code this name is only a stand-in for the device array, not a
// device address: the address is looked up per device with cudaGetSymbolAddress below.
static __device__ __align__(256) double g_tsmqr_scratch[kStripDoubles + kStatusDoubles];

// Device address of g_tsmqr_scratch per device ordinal (nullptr until that device's set-up).
// The set-up runs under g_setup_mutex, so host threads making their first call on a device
// together look the address up once; later calls read the slot without locking.
std::atomic<double *> g_scratch_addr[kMaxDevices] = {};
std::mutex g_setup_mutex;
}  // namespace

// Forgets every device's set-up (palial_gpu_finalize): the next call on a device looks the
// address up again in whatever context is current then (after a cudaDeviceReset, say).
void palial::noalloc_reset() {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    for (auto &slot : g_scratch_addr) slot.store(nullptr, std::memory_order_release);
}

extern "C" int palial_gpu_tile_dtsmqr_noalloc(int nb, double *dA1, double *dA2, const double *dV, const double *dT,
                                              int lda, void *stream) {
    if (nb <= 0 || nb % 64 != 0 || lda < nb || !dA1 || !dA2 || !dV || !dT) return PALIAL_ERR_ARG;
    if (nb > kMaxNb) return PALIAL_ERR_ARG;  // the fixed scratch covers tiles up to 512 x 512
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return PALIAL_ERR_NO_DEVICE;
    }
    if (dev < 0 || dev >= kMaxDevices) return PALIAL_ERR_ARG;
    double *scratch = g_scratch_addr[dev].load(std::memory_order_acquire);
    if (!scratch) {
        // First call on this device (which is current): find the array's device address and
        // allow the tile kernel its dynamic shared memory.  Neither step allocates memory.
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        scratch = g_scratch_addr[dev].load(std::memory_order_acquire);
        if (!scratch) {
            void *p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_tsmqr_scratch);
            if (e != cudaSuccess || !p) return PALIAL_ERR_CUDA;
            e = palial::sched_configure();
            if (e != cudaSuccess) return PALIAL_ERR_CUDA;
            scratch = static_cast<double *>(p);
            g_scratch_addr[dev].store(scratch, std::memory_order_release);
        }
    }
    // Nothing in the scratch has to start at zero: the kernel writes both strips in full
    // before reading them, and TSMQR never writes the status block.
    int *status = reinterpret_cast<int *>(scratch + kStripDoubles);
    const cudaError_t e = palial::tile_task_launch(palial::T_TSMQR, nb, lda, dA1, dA2, const_cast<double *>(dV),
                                                   const_cast<double *>(dT), scratch, status,
                                                   static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? PALIAL_OK : PALIAL_ERR_CUDA;
}
