// nvml_clock.cpp -- read-only GPU clock queries through NVML, loaded at run time.
//
// The reference controls CPU frequencies per task (palial_power/server.c:58-87); on a GPU the
// library only REPORTS clocks: the SM clock and its maximum, and the active clock-event
// (throttle) reasons.  NVML is opened with dlopen so the library has no link-time dependency
// on it; when it is missing every value is -1.  Only query functions are resolved: nothing
// here can change a clock, a power limit or any other setting.  PALIAL_NVML_LIBRARY names
// another NVML-compatible library (tests use a fake one).
#include <dlfcn.h>

#include <cstdlib>
#include <mutex>

#include "host_state.hpp"

namespace palial {

namespace {

typedef int (*fn_init)(void);
typedef int (*fn_handle_pci)(const char *, void **);
typedef int (*fn_handle_index)(unsigned, void **);
typedef int (*fn_clock)(void *, int, unsigned *);
typedef int (*fn_reasons)(void *, unsigned long long *);

constexpr int kNvmlClockSm = 1;  // nvmlClockType_t NVML_CLOCK_SM

struct Nvml {
    std::once_flag once;
    bool ok = false;
    fn_handle_pci by_pci = nullptr;
    fn_handle_index by_index = nullptr;
    fn_clock clock = nullptr, max_clock = nullptr;
    fn_reasons reasons = nullptr;
} nv;

void nvml_open() {
    const char *path = getenv("PALIAL_NVML_LIBRARY");
    void *h = dlopen(path && *path ? path : "libnvidia-ml.so.1", RTLD_NOW | RTLD_LOCAL);
    if (!h) return;
    auto init = (fn_init)dlsym(h, "nvmlInit_v2");
    nv.by_pci = (fn_handle_pci)dlsym(h, "nvmlDeviceGetHandleByPciBusId_v2");
    nv.by_index = (fn_handle_index)dlsym(h, "nvmlDeviceGetHandleByIndex_v2");
    nv.clock = (fn_clock)dlsym(h, "nvmlDeviceGetClockInfo");
    nv.max_clock = (fn_clock)dlsym(h, "nvmlDeviceGetMaxClockInfo");
    nv.reasons = (fn_reasons)dlsym(h, "nvmlDeviceGetCurrentClocksEventReasons");
    if (!nv.reasons) nv.reasons = (fn_reasons)dlsym(h, "nvmlDeviceGetCurrentClocksThrottleReasons");
    nv.ok = init && nv.clock && (nv.by_pci || nv.by_index) && init() == 0;
}

// NVML handle of the CUDA device the library uses (by PCI bus id; index 0 when the CUDA
// runtime has no device, as in CPU-only tests against a fake NVML).
void *nvml_device() {
    std::call_once(nv.once, nvml_open);
    if (!nv.ok) return nullptr;
    void *dev = nullptr;
    char bus[32];
    const int cuda_dev = g.device >= 0 ? g.device : 0;
    if (nv.by_pci && cudaDeviceGetPCIBusId(bus, sizeof bus, cuda_dev) == cudaSuccess) {
        if (nv.by_pci(bus, &dev) == 0) return dev;
    } else {
        cudaGetLastError();
    }
    if (nv.by_index && nv.by_index((unsigned)cuda_dev, &dev) == 0) return dev;
    return nullptr;
}

}  // namespace

bool nvml_sample(double *sm_mhz, double *sm_max_mhz, long long *reasons) {
    *sm_mhz = *sm_max_mhz = -1;
    *reasons = -1;
    void *dev = nvml_device();
    if (!dev) return false;
    unsigned v = 0;
    if (nv.clock(dev, kNvmlClockSm, &v) == 0) *sm_mhz = v;
    if (nv.max_clock && nv.max_clock(dev, kNvmlClockSm, &v) == 0) *sm_max_mhz = v;
    unsigned long long r = 0;
    if (nv.reasons && nv.reasons(dev, &r) == 0) *reasons = (long long)r;
    return *sm_mhz >= 0;
}

}  // namespace palial

extern "C" int palial_gpu_clock_sample(double *sm_mhz, double *sm_max_mhz, long long *reasons) {
    double a, b;
    long long r;
    const bool ok = palial::nvml_sample(&a, &b, &r);
    if (sm_mhz) *sm_mhz = a;
    if (sm_max_mhz) *sm_max_mhz = b;
    if (reasons) *reasons = r;
    return ok ? PALIAL_OK : PALIAL_ERR_NO_DEVICE;
}
