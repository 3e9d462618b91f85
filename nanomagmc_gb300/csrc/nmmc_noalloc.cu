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
#include <math.h>

#include <mutex>

#include "nmmc_internal.h"

namespace nmmc {

// Scratch of the allocation-free measurement: NMMC_STATIC_SCRATCH_DOUBLES doubles (2 MiB).
// Every GPU that loads this library holds it until the process exits. In host code the name
// is only a stand-in for the device array; its device address comes from
// cudaGetSymbolAddress, taken once per device. A call with a device chain list keeps a
// checked copy of the list at the front (256-byte aligned groups of 64 indices) and the
// measurement kernels' partial sums behind it.
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

// The caller's device list, copied with every index outside [0, nchains) replaced by chain 0,
// so that the measurement kernels only ever read the context's own chains.
__global__ void k_static_list(const int* __restrict__ in, int n, int nchains, int* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const int v = in[i];
        out[i] = (v >= 0 && v < nchains) ? v : 0;
    }
}

// Rows of out-of-range list entries: every observable (and every slice of Q) is NaN.
__global__ void k_static_poison(const int* __restrict__ in, int n, int nchains, int nslices,
                                double* __restrict__ obs, double* __restrict__ q) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int v = in[i];
    if (v >= 0 && v < nchains) return;
    for (int k = 0; k < NMMC_OBS_N; ++k) obs[(size_t)i * NMMC_OBS_N + k] = nan("");
    if (q)
        for (int k = 0; k < nslices; ++k) q[(size_t)i * nslices + k] = nan("");
}
}  // namespace

}  // namespace nmmc

using namespace nmmc;

struct nmmc_ctx : public nmmc::Ctx {};

extern "C" int nmmc_measure_static(nmmc_ctx* c, const int* d_chains, int n, double* d_obs, double* d_q) {
    if (!c || !d_obs) return set_error(NMMC_ERR_ARG, "null argument");
    if (!d_chains) n = c->nchains;
    if (n < 0) return set_error(NMMC_ERR_ARG, "chain count %d out of range", n);
    if (n == 0) return NMMC_OK;
    // a device list needs a checked copy in front of the partial sums
    const size_t list_doubles = d_chains ? ((size_t)n + 63) / 64 * 32 : 0;
    const size_t per_chain = measure_partials_per_chain(*c);
    const size_t need = list_doubles + (size_t)n * per_chain;
    if (need > NMMC_STATIC_SCRATCH_DOUBLES)
        return set_error(NMMC_ERR_ARG,
                         "%d chains need %zu doubles of static scratch; it holds %d (at most %zu chains of "
                         "this lattice per call)",
                         n, need, NMMC_STATIC_SCRATCH_DOUBLES,
                         (size_t)NMMC_STATIC_SCRATCH_DOUBLES / (per_chain + 1));
    double* scratch = nullptr;
    int rc = scratch_address(c->device, &scratch);
    if (rc) return rc;
    // changed (T, H) reach the device as one copy from the context's page-locked staging block
    // (the energy reads H in FP64)
    if ((rc = upload_params(*c))) return rc;
    const int* list = c->d_all;
    if (d_chains) {
        int* checked = reinterpret_cast<int*>(scratch);
        k_static_list<<<(n + 255) / 256, 256, 0, c->stream>>>(d_chains, n, c->nchains, checked);
        list = checked;
    }
    if ((rc = launch_measure_into(*c, list, n, scratch + list_doubles, NMMC_STATIC_SCRATCH_DOUBLES - list_doubles,
                                  d_obs, d_q)))
        return rc;
    if (d_chains)
        k_static_poison<<<(n + 255) / 256, 256, 0, c->stream>>>(d_chains, n, c->nchains, c->nslices, d_obs, d_q);
    return cuda_check(cudaGetLastError(), "static measure launch");
}
