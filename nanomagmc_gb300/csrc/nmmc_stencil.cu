// Shared-memory resident sweeps of unmasked 2-D Heisenberg lattices in their stencil layout.
//
// The general resident kernel (nmmc_resident.cu) keeps only filled sites and gives each one a
// record of neighbour indices, so that Weibull particles of any size pack densely; a site then
// costs a record decode and twelve scalar shared-memory gathers per update. An unmasked
// lattice needs neither: here each CTA holds S whole chains in the split-colour layout of HBM
// (per chain and colour three planes of ly rows of hx sites) and updates four consecutive
// same-colour sites per thread item with 16-byte shared-memory loads of the own row and of the
// other colour's rows y-1, y, y+1, exactly as the four-site HBM half-sweep does from HBM. The
// per-site arithmetic, the draw order and the Philox counters are those of the HBM kernel
// (and of the record kernel), so every path gives the same chain bit for bit. With MEASURE the
// observables of each chain are computed from the spins still in shared memory after the last
// sweep (the terms of the streaming measurement kernel, summed in FP32 per thread and warp and
// in FP64 across warps) and written with the accumulators.
#include <algorithm>

#include "nmmc_kernels.cuh"

namespace nmmc {

namespace {

constexpr int kStThreads = 768;
constexpr int kStMaxSlots = 32;

__device__ __forceinline__ float stv(const float4& v, int k) {
    return k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w));
}

// Loads of one quad from shared memory: own spins, the other colour's same row, the
// x-neighbour outside the quad and rows y +- 1 (zero where missing on an open lattice).
template <bool PERIODIC>
__device__ __forceinline__ void st_load(const DevModel& m, const float* own, const float* oth, int NH, int y,
                                        int h0, int xp, float4 (&s)[3], float4 (&same)[3], float (&ex)[3],
                                        float4 (&yp)[3], float4 (&ym)[3]) {
    const int hx = m.hx, ly = m.ly;
    const int rb = y * hx + h0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        s[c] = *reinterpret_cast<const float4*>(own + c * NH + rb);
        same[c] = *reinterpret_cast<const float4*>(oth + c * NH + rb);
    }
    int ho = xp ? h0 + 4 : h0 - 1;
    bool ok = true;
    if (PERIODIC) ho = (ho < 0) ? hx - 1 : (ho >= hx ? 0 : ho);
    else ok = ho >= 0 && ho < hx;
#pragma unroll
    for (int c = 0; c < 3; ++c) ex[c] = ok ? oth[c * NH + y * hx + ho] : 0.0f;
    int yu = y + 1, yd = y - 1;
    bool oU = true, oD = true;
    if (PERIODIC) {
        yu = (yu == ly) ? 0 : yu;
        yd = (yd < 0) ? ly - 1 : yd;
    } else {
        oU = yu < ly;
        oD = yd >= 0;
    }
    const float4 vz = {};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        yp[c] = oU ? *reinterpret_cast<const float4*>(oth + c * NH + yu * hx + h0) : vz;
        ym[c] = oD ? *reinterpret_cast<const float4*>(oth + c * NH + yd * hx + h0) : vz;
    }
}

// The four sites' neighbours in stencil order (+x, -x, +y, -y) for component c.
template <bool PERIODIC>
__device__ __forceinline__ void st_nb(const DevModel& m, const float4& same, float ex, const float4& yp,
                                      const float4& ym, int k, int h0, int xp, float (&nb)[4]) {
    const float sm = stv(same, k);
    const float sh = xp ? (k < 3 ? stv(same, k + 1) : ex) : (k > 0 ? stv(same, k - 1) : ex);
    float plusx = xp ? sh : sm, minusx = xp ? sm : sh;
    if (!PERIODIC) {
        const int x = 2 * (h0 + k) + xp;
        if (x + 1 >= m.edge) plusx = 0.0f;
        if (x == 0) minusx = 0.0f;
    }
    nb[0] = plusx;
    nb[1] = minusx;
    nb[2] = stv(yp, k);
    nb[3] = stv(ym, k);
}

}  // namespace

template <int DK, bool PERIODIC, bool MEASURE>
__global__ void __launch_bounds__(kStThreads, 1)
k_resident_stencil(const DevModel m, float* __restrict__ spins, const float4* __restrict__ bh,
                   unsigned long long* __restrict__ sweep, const int* __restrict__ chains, int n, int S,
                   int nsweeps, const double* __restrict__ Hd, double* __restrict__ obs, double* __restrict__ qout,
                   double* __restrict__ acc, int accumulate) {
    extern __shared__ __align__(16) float st_sm[];
    __shared__ float4 sp[kStMaxSlots];
    __shared__ unsigned long long ssw[kStMaxSlots];
    __shared__ int sch[kStMaxSlots];
    __shared__ float wred[kStThreads / 32][kNP];
    const int NH = m.nhalf;                 // sites per colour plane (hx * ly)
    const size_t P = (size_t)m.nhalf_pad;
    const int hx = m.hx, qpr = hx >> 2, Q = qpr * m.ly;
    const int c0 = blockIdx.x * S;
    const int ns = min(S, n - c0);
    if (ns <= 0) return;
    const int tid = threadIdx.x;
    for (int t = tid; t < ns; t += blockDim.x) {
        const int ch = chains[c0 + t];
        sch[t] = ch;
        sp[t] = bh[ch];
        ssw[t] = sweep[ch];
    }
    __syncthreads();
    const int nv = NH >> 2;                 // float4 per plane
    for (int i = tid; i < ns * 6 * nv; i += blockDim.x) {
        const int sl = i / (6 * nv), r = i - sl * 6 * nv, pl = r / nv, j = r - pl * nv;
        reinterpret_cast<float4*>(st_sm)[(size_t)(sl * 6 + pl) * nv + j] =
            __ldg(reinterpret_cast<const float4*>(spins + ((size_t)sch[sl] * 6 + pl) * P) + j);
    }
    __syncthreads();
    const int qshift = m.qpr_shift;         // log2(hx / 4) or -1
    const int Qs = (Q & (Q - 1)) == 0 ? __ffs(Q) - 1 : -1;   // log2(Q) or -1
    for (int sw = 0; sw < nsweeps; ++sw) {
        for (int colour = 0; colour < 2; ++colour) {
            for (int it = tid; it < ns * Q; it += blockDim.x) {
                const int sl = Qs >= 0 ? (it >> Qs) : (it / Q), r = it - sl * Q;
                const int y = qshift >= 0 ? (r >> qshift) : (r / qpr);
                const int h0 = (r - y * qpr) * 4;
                const int xp = (y + colour) & 1;
                float* own = st_sm + (size_t)(sl * 6 + colour * 3) * NH;
                const float* oth = st_sm + (size_t)(sl * 6 + (colour ^ 1) * 3) * NH;
                float4 s[3], same[3], yp[3], ym[3];
                float ex[3];
                st_load<PERIODIC>(m, own, oth, NH, y, h0, xp, s, same, ex, yp, ym);
                const int chain = sch[sl];
                const float4 p = sp[sl];
                const unsigned long long swc = ssw[sl] + (unsigned)sw;
                const uint32_t boxrow = (uint32_t)(m.edge * y);
                nmmc_u4 rnext = sweep_draw<true>(m, boxrow + (uint32_t)(2 * h0 + xp), swc, (uint32_t)chain);
                float out[3][4];
                bool any = false;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    float nx[4], ny[4], nz[4];
                    st_nb<PERIODIC>(m, same[0], ex[0], yp[0], ym[0], k, h0, xp, nx);
                    st_nb<PERIODIC>(m, same[1], ex[1], yp[1], ym[1], k, h0, xp, ny);
                    st_nb<PERIODIC>(m, same[2], ex[2], yp[2], ym[2], k, h0, xp, nz);
                    const float sx = stv(s[0], k), sy = stv(s[1], k), sz = stv(s[2], k);
                    const nmmc_u4 rr = rnext;
                    if (k < 3)
                        rnext = sweep_draw<true>(m, boxrow + (uint32_t)(2 * (h0 + k + 1) + xp), swc, (uint32_t)chain);
                    float hxf, hyf, hzf, tx, ty, tz;
                    heis_field<4, DK>(m, nx, ny, nz, p, hxf, hyf, hzf);
                    const bool a = heis_try(hxf, hyf, hzf, sx, sy, sz, p, rr, tx, ty, tz);
                    out[0][k] = a ? tx : sx;
                    out[1][k] = a ? ty : sy;
                    out[2][k] = a ? tz : sz;
                    any |= a;
                }
                if (any) {
#pragma unroll
                    for (int c = 0; c < 3; ++c)
                        *reinterpret_cast<float4*>(own + c * NH + y * hx + h0) =
                            make_float4(out[c][0], out[c][1], out[c][2], out[c][3]);
                }
            }
            __syncthreads();
        }
    }
    if constexpr (MEASURE) {
        // per chain: the streaming measurement kernel's per-site terms (Old/lib/thermodynamics.cpp:
        // 71-221) over both colours, FP32 per thread and warp, FP64 across warps in warp order
        const int lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
        const bool pq = PERIODIC && m.periodic_q;
        const int e4 = m.edge - m.edge % 4;
        for (int sl = 0; sl < ns; ++sl) {
            float a[kNP];
#pragma unroll
            for (int k = 0; k < kNP; ++k) a[k] = 0.0f;
            for (int it = tid; it < 2 * Q; it += blockDim.x) {
                const int colour = it & 1, r = it >> 1;
                const int y = qshift >= 0 ? (r >> qshift) : (r / qpr);
                const int h0 = (r - y * qpr) * 4;
                const int xp = (y + colour) & 1;
                const float* own = st_sm + (size_t)(sl * 6 + colour * 3) * NH;
                const float* oth = st_sm + (size_t)(sl * 6 + (colour ^ 1) * 3) * NH;
                float4 s[3], same[3], yp[3], ym[3];
                float ex[3];
                st_load<PERIODIC>(m, own, oth, NH, y, h0, xp, s, same, ex, yp, ym);
                const bool qyu = (y + 1 < m.edge || pq) && (PERIODIC || y + 1 < m.ly);
                const bool qyd = (y >= 1 || pq);
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const int x = 2 * (h0 + k) + xp;
                    float n0[4], n1[4], n2[4];
                    st_nb<PERIODIC>(m, same[0], ex[0], yp[0], ym[0], k, h0, xp, n0);
                    st_nb<PERIODIC>(m, same[1], ex[1], yp[1], ym[1], k, h0, xp, n1);
                    st_nb<PERIODIC>(m, same[2], ex[2], yp[2], ym[2], k, h0, xp, n2);
                    const float s0 = stv(s[0], k), s1 = stv(s[1], k), s2 = stv(s[2], k);
                    float f0 = 0.f, f1 = 0.f, f2 = 0.f;
                    if (DK <= kDmiGeneral) {
#pragma unroll
                        for (int d = 0; d < 4; ++d) {
                            const float J = m.J[d];
                            f0 = fmaf(J, n0[d], f0);
                            f1 = fmaf(J, n1[d], f1);
                            f2 = fmaf(J, n2[d], f2);
                            if (DK == kDmiGeneral) {
                                f0 = fmaf(m.De[d][1], n2[d], fmaf(-m.De[d][2], n1[d], f0));
                                f1 = fmaf(m.De[d][2], n0[d], fmaf(-m.De[d][0], n2[d], f1));
                                f2 = fmaf(m.De[d][0], n1[d], fmaf(-m.De[d][1], n0[d], f2));
                            }
                        }
                    } else {
#pragma unroll
                        for (int ax = 0; ax < 2; ++ax) {
                            const int kp = 2 * ax, km = 2 * ax + 1;
                            const float J = m.J[kp];
                            f0 = fmaf(J, n0[kp] + n0[km], f0);
                            f1 = fmaf(J, n1[kp] + n1[km], f1);
                            f2 = fmaf(J, n2[kp] + n2[km], f2);
                            const float d0 = n0[kp] - n0[km], d1 = n1[kp] - n1[km], d2 = n2[kp] - n2[km];
                            if (DK == kDmiPairs) {
                                f0 = fmaf(m.De[kp][1], d2, fmaf(-m.De[kp][2], d1, f0));
                                f1 = fmaf(m.De[kp][2], d0, fmaf(-m.De[kp][0], d2, f1));
                                f2 = fmaf(m.De[kp][0], d1, fmaf(-m.De[kp][1], d0, f2));
                            } else {
                                const float D = m.De[kp][ax];
                                if (ax == 0) {
                                    f1 = fmaf(-D, d2, f1);
                                    f2 = fmaf(D, d1, f2);
                                } else {
                                    f0 = fmaf(D, d2, f0);
                                    f2 = fmaf(-D, d0, f2);
                                }
                            }
                        }
                    }
                    a[0] = fmaf(s0, f0, fmaf(s1, f1, fmaf(s2, f2, a[0])));
                    a[1] += s0;
                    a[2] += s1;
                    a[3] += s2;
                    if (colour == 0) {
                        a[4] += s0;
                        a[5] += s1;
                        a[6] += s2;
                    }
                    const int possum = x + y, posdiff = -x + y + e4;
                    if (possum % 4 == 0 && posdiff % 4 == 0) {
                        a[7] += s0;
                        a[8] += s1;
                        a[9] += s2;
                    }
                    const bool qxm = (x >= 1 || pq), qxp = (x + 1 < m.edge || pq);
                    if (qxm && qyu) a[10] += solid_angle_f(s0, s1, s2, n0[1], n1[1], n2[1], n0[2], n1[2], n2[2]);
                    if (qxp && qyd) a[10] += solid_angle_f(s0, s1, s2, n0[0], n1[0], n2[0], n0[3], n1[3], n2[3]);
                }
            }
#pragma unroll
            for (int k = 0; k < kNP; ++k) {
                float v = a[k];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
                if (lane == 0) wred[warp][k] = v;
            }
            __syncthreads();
            if (warp == 0) {
                double v = 0.0;
                if (lane < kNP)
                    for (int w = 0; w < nw; ++w) v += (double)wred[w][lane];
                const int ch = sch[sl], ci = c0 + sl;
                const double qv = __shfl_sync(0xffffffffu, v, 10) / (2 * M_PI);
                if (qout && lane == 0) qout[ci] = qv;
                finalize_chain_warp(v, lane, Hd + 3 * (size_t)ch, qv, obs + (size_t)ci * NMMC_OBS_N,
                                    acc + (size_t)ch * NMMC_ACC_N, accumulate);
            }
            __syncthreads();
        }
    }
    for (int i = tid; i < ns * 6 * nv; i += blockDim.x) {
        const int sl = i / (6 * nv), r = i - sl * 6 * nv, pl = r / nv, j = r - pl * nv;
        reinterpret_cast<float4*>(spins + ((size_t)sch[sl] * 6 + pl) * P)[j] =
            reinterpret_cast<const float4*>(st_sm)[(size_t)(sl * 6 + pl) * nv + j];
    }
    for (int t = tid; t < ns; t += blockDim.x) sweep[sch[t]] += (unsigned long long)nsweeps;
}

// ------------------------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------------------------
// Bytes of one chain in shared memory (6 planes of hx * ly floats), or 0 when the lattice is not
// covered: unmasked 2-D Heisenberg lattices with rows of a multiple of 4 sites per colour and
// the checkerboard's axis tables.
size_t stencil_chain_bytes(const Ctx& c) {
    if (c.ising || c.masked || c.m.general || c.dim != 2 || (c.m.hx % 4) != 0) return 0;
    return (size_t)6 * c.m.nhalf * sizeof(float);
}

// Chains per CTA for a call on n chains: spread over the SMs, as many as the shared memory
// holds (0: not even one).
int stencil_slots(const Ctx& c, int n) {
    const size_t cb = stencil_chain_bytes(c);
    if (cb == 0 || n <= 0) return 0;
    const size_t static_bytes = kStMaxSlots * (sizeof(float4) + sizeof(unsigned long long) + sizeof(int)) +
                                (kStThreads / 32) * kNP * sizeof(float) + 64;
    if (c.smem_optin <= static_bytes) return 0;
    const int fit = (int)std::min<size_t>(kStMaxSlots, (c.smem_optin - static_bytes) / cb);
    if (fit < 1) return 0;
    const int spread = (n + c.sm_count - 1) / c.sm_count;
    return std::min(fit, std::max(1, spread));
}

template <int DK, bool PERIODIC, bool MEASURE>
static int stencil_launch_t(Ctx& c, const int* d_chains, int n, int nsweeps, int accumulate) {
    const int S = stencil_slots(c, n);
    if (S < 1) return set_error(NMMC_ERR_UNSUPPORTED, "lattice does not fit the stencil resident kernel");
    const size_t smem = (size_t)S * stencil_chain_bytes(c);
    auto kern = k_resident_stencil<DK, PERIODIC, MEASURE>;
    size_t& set = c.stencil_smem[DK * 4 + (PERIODIC ? 2 : 0) + (MEASURE ? 1 : 0)];
    if (set < smem) {   // raised once per kernel and context to the largest size launched
        const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return cuda_check(e, "stencil kernel shared memory");
        set = smem;
    }
    const int grid = (n + S - 1) / S;
    // a width that gives every thread the same number of quads per half-sweep
    const int items = S * (c.m.hx / 4) * c.m.ly;
    const int per = (items + kStThreads - 1) / kStThreads;
    const int threads = std::max(32, ((items + per - 1) / per + 31) / 32 * 32);
    kern<<<grid, threads, smem, c.stream>>>(c.m, (float*)c.d_spins, c.d_bh, c.d_sweep, d_chains, n, S, nsweeps,
                                            c.d_Hd, c.d_obs, c.d_q, c.d_acc, accumulate);
    return cuda_check(cudaGetLastError(), "k_resident_stencil");
}

template <bool PERIODIC, bool MEASURE>
static int stencil_launch_d(Ctx& c, const int* d_chains, int n, int nsweeps, int accumulate) {
    switch (c.m.dmi_kind) {
        case kDmiNone: return stencil_launch_t<kDmiNone, PERIODIC, MEASURE>(c, d_chains, n, nsweeps, accumulate);
        case kDmiGeneral: return stencil_launch_t<kDmiGeneral, PERIODIC, MEASURE>(c, d_chains, n, nsweeps, accumulate);
        case kDmiPairs: return stencil_launch_t<kDmiPairs, PERIODIC, MEASURE>(c, d_chains, n, nsweeps, accumulate);
        default: return stencil_launch_t<kDmiAxial, PERIODIC, MEASURE>(c, d_chains, n, nsweeps, accumulate);
    }
}

// nsweeps sweeps of the listed chains (d_chains, n entries, each chain at most once) and, with
// measure, their observables in list order and (accumulate) their accumulators.
int launch_stencil_sweeps(Ctx& c, const int* d_chains, int n, int nsweeps, bool measure, int accumulate) {
    if (n <= 0) return NMMC_OK;
    if (c.periodic) return measure ? stencil_launch_d<true, true>(c, d_chains, n, nsweeps, accumulate)
                                   : stencil_launch_d<true, false>(c, d_chains, n, nsweeps, accumulate);
    return measure ? stencil_launch_d<false, true>(c, d_chains, n, nsweeps, accumulate)
                   : stencil_launch_d<false, false>(c, d_chains, n, nsweeps, accumulate);
}

}  // namespace nmmc
