// nmmc_measure_static: the observables of nmmc_measure for callers that cannot allocate
// device memory.
//
// Who cannot allocate: code that runs while a CUDA stream is being captured into a graph
// (cudaMalloc is refused during capture), host frameworks that hand out device memory from
// their own pool or arena and forbid the CUDA allocator, and latency-critical loops where
// cudaMalloc's implicit device-wide synchronisation would stall other streams. nmmc_measure
// may allocate (it grows its partial-sum buffer on first use for a chain count); this entry
// point never does: the measurement kernels' per-block partial sums go to the fixed array
// below, and the results go to device buffers the caller owns.
#include <mutex>

#include "nmmc_internal.h"

namespace nmmc {

// Partial-sum scratch of the measurement kernels: NMMC_STATIC_SCRATCH_DOUBLES doubles (1 MiB).
// Every GPU that loads this library holds it until the process exits. In host code the name
// is only a stand-in for the device array; its device address comes from
// cudaGetSymbolAddress, taken once per device.
static __device__ __align__(256) double g_measure_scratch[NMMC_STATIC_SCRATCH_DOUBLES];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_mu;
double* g_scratch_addr[kMaxDevices] = {};

// Address of the scratch array on `dev`, looked up on the first call for that device with
// `dev` current. The caller's current device is restored.
int scratch_address(int dev, double** out) {
    if (dev < 0 || dev >= kMaxDevices) return set_error(NMMC_ERR_ARG, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_addr[dev]) {
        int prev = 0;
        cudaError_t e = cudaGetDevice(&prev);
        if (e != cudaSuccess) return cuda_check(e, "cudaGetDevice");
        if (prev != dev && (e = cudaSetDevice(dev)) != cudaSuccess) return cuda_check(e, "cudaSetDevice");
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_measure_scratch);
        if (prev != dev) cudaSetDevice(prev);
        if (e != cudaSuccess) return cuda_check(e, "cudaGetSymbolAddress(g_measure_scratch)");
        g_scratch_addr[dev] = static_cast<double*>(p);
    }
    *out = g_scratch_addr[dev];
    return NMMC_OK;
}
}  // namespace

}  // namespace nmmc

using namespace nmmc;

struct nmmc_ctx : public nmmc::Ctx {};

extern "C" int nmmc_measure_static(nmmc_ctx* c, const int* d_chains, int n, double* d_obs, double* d_q) {
    if (!c || !d_obs) return set_error(NMMC_ERR_ARG, "null argument");
    if (!d_chains) n = c->nchains;
    if (n <= 0 || n > c->nchains) return set_error(NMMC_ERR_ARG, "chain count %d out of range", n);
    double* scratch = nullptr;
    int rc = scratch_address(c->device, &scratch);
    if (rc) return rc;
    if (c->params_dirty) {
        // the energy reads H in FP64: refresh the changed chains' field values in place
        // (pageable single-value copies; no buffer is allocated). The FP32 sweep
        // parameters stay marked for the next sweep's upload.
        const int hi = c->ising ? 0 : 2;
        for (int i = 0; i < c->nchains; ++i)
            NMMC_CUDA(cudaMemcpyAsync(c->d_Hd + 3 * (size_t)i + hi, &c->H[i], sizeof(double),
                                      cudaMemcpyHostToDevice, c->stream));
    }
    return launch_measure_into(*c, d_chains ? d_chains : c->d_all, n, scratch, NMMC_STATIC_SCRATCH_DOUBLES,
                               d_obs, d_q);
}
