// Four-site half-sweep with the next quad's spins prefetched into shared memory.
//
// The four-site half-sweep (k_heis_half_q4) gives each thread one quad: it loads the quad's 21
// vectors (own spins, the other colour's same row, rows y +- 1 and z +- 1) and then computes,
// so each warp alternates between waiting on DRAM and computing, and at 3 CTAs per SM the SM
// often has no warp ready. Here each thread walks a strided sequence of quads and, before it
// computes quad i, asks for the vectors of quad i+1 with cp.async into its own slots of shared
// memory (vector-major: slot [j][thread], so a warp's accesses are contiguous); when it has
// computed quad i it waits for its own copies only (cp.async.wait_all: no barrier, no other
// thread involved), moves them to registers and continues. The per-site arithmetic, the draw
// order and the Philox counters are those of the four-site kernel, so the chain is the same
// bit for bit. Quads of one colour never overlap, and the other colour is read-only during the
// launch, so prefetching a quad early reads the values the four-site kernel reads.
#include <algorithm>

#include "nmmc_kernels.cuh"

namespace nmmc {

namespace {

constexpr int kPfThreads = 256;

__device__ __forceinline__ float pel(const float4& v, int k) {
    return k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w));
}

__device__ __forceinline__ uint32_t pf_smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// 16 (or 4) bytes from global to shared memory through L1; src_bytes 0 writes zeros (the
// source is then not read).
__device__ __forceinline__ void cp16(uint32_t dst, const void* src, int src_bytes) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp4(uint32_t dst, const void* src, int src_bytes) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}

// Where a quad sits: chain (by list position), row, first compact site, x parity.
struct QuadPos {
    int chain, y, z, h0, xp, row;
};

template <int DIM>
__device__ __forceinline__ QuadPos quad_pos(const DevModel& m, const int* __restrict__ chains, long long q, int qpc,
                                            int qpc_shift, int colour) {
    QuadPos p;
    const int ci = qpc_shift >= 0 ? (int)(q >> qpc_shift) : (int)(q / qpc);
    const int r = (int)(q - (long long)ci * qpc);
    p.chain = chains[ci];
    const int qpr = m.hx >> 2;
    p.row = m.qpr_shift >= 0 ? (r >> m.qpr_shift) : (r / qpr);
    p.h0 = (r - p.row * qpr) * 4;
    if (DIM == 3) {
        p.z = m.ly_shift >= 0 ? (p.row >> m.ly_shift) : (p.row / m.ly);
        p.y = p.row - p.z * m.ly;
    } else {
        p.z = 0;
        p.y = p.row;
    }
    p.xp = (p.y + p.z + colour) & 1;
    return p;
}

// Slots of one thread: vectors 0-2 own spins, 3-5 same row, 6-8 row y+1, 9-11 row y-1,
// 12-14 plane z+1, 15-17 plane z-1 (3-D); scalars 0-2 the x-neighbour outside the quad.
template <int DIM, bool PERIODIC>
__device__ __forceinline__ void issue_quad(const DevModel& m, const float* __restrict__ spins, const QuadPos& p,
                                           int colour, uint32_t vbase, uint32_t sbase) {
    const size_t P = (size_t)m.nhalf_pad;
    const float* own = spins + ((size_t)p.chain * 2 + colour) * 3 * P;
    const float* oth = spins + ((size_t)p.chain * 2 + (colour ^ 1)) * 3 * P;
    const int rb = p.row * m.hx + p.h0;
    constexpr uint32_t kStride = kPfThreads * 16;   // bytes between slots j and j+1 of a thread
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        cp16(vbase + (0 + c) * kStride, own + c * P + rb, 16);
        cp16(vbase + (3 + c) * kStride, oth + c * P + rb, 16);
    }
    int hx_out = p.xp ? p.h0 + 4 : p.h0 - 1;
    bool ex_ok = true;
    if (PERIODIC) hx_out = (hx_out < 0) ? m.hx - 1 : (hx_out >= m.hx ? 0 : hx_out);
    else {
        ex_ok = hx_out >= 0 && hx_out < m.hx;
        if (!ex_ok) hx_out = p.h0;
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) cp4(sbase + c * kPfThreads * 4, oth + c * P + p.row * m.hx + hx_out, ex_ok ? 4 : 0);
    int yu = p.y + 1, yd = p.y - 1;
    bool okU = true, okD = true;
    if (PERIODIC) {
        yu = (yu == m.edge) ? 0 : yu;
        yd = (yd < 0) ? m.edge - 1 : yd;
    } else {
        okU = yu < m.edge;
        okD = yd >= 0;
        if (!okU) yu = p.y;
        if (!okD) yd = p.y;
    }
    const int ru = (p.z * m.ly + yu) * m.hx + p.h0, rd = (p.z * m.ly + yd) * m.hx + p.h0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        cp16(vbase + (6 + c) * kStride, oth + c * P + ru, okU ? 16 : 0);
        cp16(vbase + (9 + c) * kStride, oth + c * P + rd, okD ? 16 : 0);
    }
    if (DIM == 3) {
        int zu = p.z + 1, zd = p.z - 1;
        bool oU = true, oD = true;
        if (PERIODIC) {
            zu = (zu == m.edge) ? 0 : zu;
            zd = (zd < 0) ? m.edge - 1 : zd;
        } else {
            oU = zu < m.lz;
            oD = zd >= 0;
            if (!oU) zu = p.z;
            if (!oD) zd = p.z;
        }
        const int rzu = (zu * m.ly + p.y) * m.hx + p.h0, rzd = (zd * m.ly + p.y) * m.hx + p.h0;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            cp16(vbase + (12 + c) * kStride, oth + c * P + rzu, oU ? 16 : 0);
            cp16(vbase + (15 + c) * kStride, oth + c * P + rzd, oD ? 16 : 0);
        }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}

}  // namespace

template <int DIM, bool PERIODIC, int DK>
__global__ void __launch_bounds__(kPfThreads, 2)
k_heis_half_pf(const DevModel m, float* __restrict__ spins, const float4* __restrict__ bh,
               const unsigned long long* __restrict__ sweep, const int* __restrict__ chains, int colour,
               unsigned sweep_off, long long nquads, int qpc, int qpc_shift) {
    constexpr int NV = DIM == 3 ? 18 : 12;
    constexpr int ND = 2 * DIM;
    extern __shared__ float4 pf_vec[];   // [NV][kPfThreads] float4, then [3][kPfThreads] float
    float* pf_sc = reinterpret_cast<float*>(pf_vec + NV * kPfThreads);
    const int tid = threadIdx.x;
    const uint32_t vbase = pf_smem_u32(pf_vec + tid), sbase = pf_smem_u32(pf_sc + tid);
    const long long G = (long long)gridDim.x * kPfThreads;
    long long q = (long long)blockIdx.x * kPfThreads + tid;
    if (q >= nquads) return;
    QuadPos pos = quad_pos<DIM>(m, chains, q, qpc, qpc_shift, colour);
    issue_quad<DIM, PERIODIC>(m, spins, pos, colour, vbase, sbase);
    const size_t P = (size_t)m.nhalf_pad;
    while (true) {
        asm volatile("cp.async.wait_all;" ::: "memory");
        float4 v[NV];
        float ex[3];
#pragma unroll
        for (int j = 0; j < NV; ++j) v[j] = pf_vec[j * kPfThreads + tid];
#pragma unroll
        for (int c = 0; c < 3; ++c) ex[c] = pf_sc[c * kPfThreads + tid];
        const QuadPos cur = pos;
        const long long qn = q + G;
        const bool more = qn < nquads;
        if (more) {   // the next quad's copies run while this quad is computed
            pos = quad_pos<DIM>(m, chains, qn, qpc, qpc_shift, colour);
            issue_quad<DIM, PERIODIC>(m, spins, pos, colour, vbase, sbase);
        }
        // ---- the four-site kernel's arithmetic on quad `cur` ----
        const float4 p = bh[cur.chain];
        const unsigned long long sw = sweep[cur.chain] + sweep_off;
        const uint32_t boxrow = (uint32_t)(m.edge * (cur.y + m.edge * cur.z));
        const int xp = cur.xp, h0 = cur.h0;
        bool any = false;
        nmmc_u4 rnext = sweep_draw<true>(m, boxrow + (uint32_t)(2 * h0 + xp), sw, (uint32_t)cur.chain);
        float out[3][4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            float nx[ND], ny[ND], nz[ND];
            float* nn[3] = {nx, ny, nz};
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float sm = pel(v[3 + c], k);
                const float sh = xp ? (k < 3 ? pel(v[3 + c], k + 1) : ex[c]) : (k > 0 ? pel(v[3 + c], k - 1) : ex[c]);
                float plusx = xp ? sh : sm, minusx = xp ? sm : sh;
                if (!PERIODIC) {
                    const int x = 2 * (h0 + k) + xp;
                    if (x + 1 >= m.edge) plusx = 0.0f;
                    if (x == 0) minusx = 0.0f;
                }
                nn[c][0] = plusx;
                nn[c][1] = minusx;
                nn[c][2] = pel(v[6 + c], k);
                nn[c][3] = pel(v[9 + c], k);
                if (DIM == 3) {
                    nn[c][4] = pel(v[(DIM == 3 ? 12 : 0) + c], k);
                    nn[c][5] = pel(v[(DIM == 3 ? 15 : 0) + c], k);
                }
            }
            const float sx = pel(v[0], k), sy = pel(v[1], k), sz = pel(v[2], k);
            float tx, ty, tz;
            const nmmc_u4 r = rnext;
            if (k < 3) rnext = sweep_draw<true>(m, boxrow + (uint32_t)(2 * (h0 + k + 1) + xp), sw, (uint32_t)cur.chain);
            float hx, hy, hz;
            heis_field<ND, DK>(m, nx, ny, nz, p, hx, hy, hz);
            const bool acc = heis_try(hx, hy, hz, sx, sy, sz, p, r, tx, ty, tz);
            out[0][k] = acc ? tx : sx;
            out[1][k] = acc ? ty : sy;
            out[2][k] = acc ? tz : sz;
            any |= acc;
        }
        if (any) {
            float* own = spins + ((size_t)cur.chain * 2 + colour) * 3 * P;
            const int rb = cur.row * m.hx + h0;
#pragma unroll
            for (int c = 0; c < 3; ++c)
                *reinterpret_cast<float4*>(own + c * P + rb) = make_float4(out[c][0], out[c][1], out[c][2], out[c][3]);
        }
        if (!more) break;
        q = qn;
    }
}

// Lattices the kernel covers: those of the four-site kernel (unmasked Heisenberg, rows of a
// multiple of 4 sites per colour).
static size_t pf_smem(int dim) { return (size_t)((dim == 3 ? 18 : 12) * 16 + 3 * 4) * kPfThreads; }

template <int DIM, bool PERIODIC, int DK>
static int pf_launch_t(Ctx& c, const int* d_chains, int n, int colour, unsigned off) {
    auto kern = k_heis_half_pf<DIM, PERIODIC, DK>;
    const size_t smem = pf_smem(DIM);
    int& per_sm = c.pf_per_sm[(DIM == 3 ? 8 : 0) + DK * 2 + (PERIODIC ? 1 : 0)];
    if (per_sm == 0) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return cuda_check(e, "prefetching half-sweep shared memory");
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kPfThreads, smem);
        if (e != cudaSuccess) return cuda_check(e, "prefetching half-sweep occupancy");
        if (per_sm < 1) {
            per_sm = 0;
            return set_error(NMMC_ERR_CUDA, "prefetching half-sweep does not fit on an SM");
        }
    }
    const int qpc = (c.m.hx / 4) * c.m.ly * c.m.lz;
    int qpc_shift = -1;
    for (int s = 0; s < 31; ++s)
        if ((1 << s) == qpc) qpc_shift = s;
    const long long nquads = (long long)n * qpc;
    const long long grid = std::min<long long>((long long)per_sm * c.sm_count, (nquads + kPfThreads - 1) / kPfThreads);
    if (grid < 1) return NMMC_OK;
    kern<<<(unsigned)grid, kPfThreads, smem, c.stream>>>(c.m, (float*)c.d_spins, c.d_bh, c.d_sweep, d_chains, colour,
                                                         off, nquads, qpc, qpc_shift);
    return cuda_check(cudaGetLastError(), "k_heis_half_pf");
}

template <int DIM, bool PERIODIC>
static int pf_launch_d(Ctx& c, const int* d_chains, int n, int colour, unsigned off) {
    switch (c.m.dmi_kind) {
        case kDmiNone: return pf_launch_t<DIM, PERIODIC, kDmiNone>(c, d_chains, n, colour, off);
        case kDmiGeneral: return pf_launch_t<DIM, PERIODIC, kDmiGeneral>(c, d_chains, n, colour, off);
        case kDmiPairs: return pf_launch_t<DIM, PERIODIC, kDmiPairs>(c, d_chains, n, colour, off);
        default: return pf_launch_t<DIM, PERIODIC, kDmiAxial>(c, d_chains, n, colour, off);
    }
}

int launch_pf_half(Ctx& c, const int* d_chains, int n, int colour, unsigned off) {
    if (c.dim == 3) return c.periodic ? pf_launch_d<3, true>(c, d_chains, n, colour, off)
                                      : pf_launch_d<3, false>(c, d_chains, n, colour, off);
    return c.periodic ? pf_launch_d<2, true>(c, d_chains, n, colour, off) : pf_launch_d<2, false>(c, d_chains, n, colour, off);
}

}  // namespace nmmc
