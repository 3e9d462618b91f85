// HBM-streaming checkerboard half-sweeps, observables, dE probes, the FP64 sequential
// replay, random starts and counter bookkeeping.
//
// Hot path: state::equil (Old/lib/state.cpp:171-203) becomes two half-sweep launches per
// sweep, one per colour of the checkerboard. Each thread updates one site of the active
// colour: it reads its own spin and its 2*dim neighbours (all of the other colour, so no
// thread reads a spin another thread of the same launch writes), draws one Philox4x32-10
// block keyed by (box index, sweep, chain) and applies the reference's dE and acceptance
// rule (Old/lib/thermodynamics.cpp:51-69, state.cpp:190-201) in FP32.
#include <math.h>

#include "nmmc_kernels.cuh"

namespace nmmc {

// ------------------------------------------------------------------------------------------
// Half-sweep kernels
// ------------------------------------------------------------------------------------------
template <int DIM, bool PERIODIC, bool MASKED, int DK>
__global__ void __launch_bounds__(256)
k_heis_half(const DevModel m, float* __restrict__ spins, const uint32_t* __restrict__ fill,
            const int* __restrict__ fill_n, const float4* __restrict__ bh,
            const unsigned long long* __restrict__ sweep, const int* __restrict__ chains, int colour,
            unsigned sweep_off) {
    const int chain = chains[blockIdx.y];
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (MASKED) {   // thread j: the chain's j-th filled site of this colour
        const int seg = chain * 2 + colour;
        if (i >= fill_n[seg]) return;
        i = (int)__ldg(&fill[(size_t)seg * m.nhalf + i]);
    } else if (i >= m.nhalf) {
        return;
    }
    int x, y, z;
    decode_site<DIM>(m, i, colour, x, y, z);
    const size_t P = (size_t)m.nhalf_pad;
    if (!MASKED && x >= m.edge) return;
    float* own = spins + ((size_t)chain * 2 + colour) * 3 * P;
    const float* oth = spins + ((size_t)chain * 2 + (colour ^ 1)) * 3 * P;
    constexpr int ND = 2 * DIM;
    float nx[ND], ny[ND], nz[ND];
#pragma unroll
    for (int k = 0; k < ND; ++k) {
        int j = nb_compact<PERIODIC>(m, x, y, z, k);
        if (PERIODIC || j >= 0) {
            nx[k] = __ldg(oth + j);
            ny[k] = __ldg(oth + P + j);
            nz[k] = __ldg(oth + 2 * P + j);
        } else {
            nx[k] = ny[k] = nz[k] = 0.0f;
        }
    }
    const float sx = own[i], sy = own[P + i], sz = own[2 * P + i];
    const float4 p = bh[chain];
    const uint32_t box = (uint32_t)(x + m.edge * (y + m.edge * z));
    const nmmc_u4 r = sweep_draw(m, box, sweep[chain] + sweep_off, (uint32_t)chain);
    float tx, ty, tz;
    if (heis_attempt<ND, DK>(m, sx, sy, sz, nx, ny, nz, p, r, tx, ty, tz)) {
        own[i] = tx;
        own[P + i] = ty;
        own[2 * P + i] = tz;
    }
}

template <int DIM, bool PERIODIC, bool MASKED>
__global__ void __launch_bounds__(256)
k_ising_half(const DevModel m, int8_t* __restrict__ spins, const uint32_t* __restrict__ fill,
             const int* __restrict__ fill_n, const float4* __restrict__ bh,
             const unsigned long long* __restrict__ sweep, const int* __restrict__ chains, int colour,
             unsigned sweep_off) {
    const int chain = chains[blockIdx.y];
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (MASKED) {   // thread j: the chain's j-th filled site of this colour
        const int seg = chain * 2 + colour;
        if (i >= fill_n[seg]) return;
        i = (int)__ldg(&fill[(size_t)seg * m.nhalf + i]);
    } else if (i >= m.nhalf) {
        return;
    }
    int x, y, z;
    decode_site<DIM>(m, i, colour, x, y, z);
    const size_t P = (size_t)m.nhalf_pad;
    if (!MASKED && x >= m.edge) return;
    int8_t* own = spins + ((size_t)chain * 2 + colour) * P;
    const int8_t* oth = spins + ((size_t)chain * 2 + (colour ^ 1)) * P;
    constexpr int ND = 2 * DIM;
    float n[ND];
#pragma unroll
    for (int k = 0; k < ND; ++k) {
        int j = nb_compact<PERIODIC>(m, x, y, z, k);
        n[k] = (PERIODIC || j >= 0) ? (float)__ldg(oth + j) : 0.0f;
    }
    const float4 p = bh[chain];
    const uint32_t box = (uint32_t)(x + m.edge * (y + m.edge * z));
    const nmmc_u4 r = sweep_draw(m, box, sweep[chain] + sweep_off, (uint32_t)chain);
    float t;
    if (ising_attempt<ND>(m, (float)own[i], n, p, r, t)) own[i] = (int8_t)t;
}

// Masked Heisenberg lattices, compact form: thread j of chain c and colour p updates the j-th
// filled site, whose spin is entry j of the compact planes and whose table entry gives its
// neighbours' entries in the other colour (empty sites read as spin 0) in stencil order and
// its box index (the Philox counter). The same update as k_heis_half on the same values, so
// the same chain; the compact planes are dense, so the loads use whole sectors. PACKED: one
// int4 per site, neighbours as 16-bit differences to j; otherwise two int4 of absolute indices.
constexpr int kNoNeighbour16 = -32768;

// Table entry of compact site j of segment seg: the six neighbour indices (-1: none) and the
// box index.
template <bool PACKED>
__device__ __forceinline__ void compact_entry(const int4* __restrict__ tab, int seg, size_t NH, int j, int (&nbi)[6],
                                              uint32_t& box) {
    if (PACKED) {
        const int4 t = __ldg(&tab[(size_t)seg * NH + j]);
        const int w[3] = {t.x, t.y, t.z};
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            const int d = (k & 1) ? (w[k >> 1] >> 16) : (int)(short)(w[k >> 1] & 0xFFFF);
            nbi[k] = (d == kNoNeighbour16) ? -1 : j + d;
        }
        box = (uint32_t)t.w;
    } else {
        const int4 t0 = __ldg(&tab[((size_t)seg * NH + j) * 2]);
        const int4 t1 = __ldg(&tab[((size_t)seg * NH + j) * 2 + 1]);
        nbi[0] = t0.x; nbi[1] = t0.y; nbi[2] = t0.z; nbi[3] = t0.w; nbi[4] = t1.x; nbi[5] = t1.y;
        box = (uint32_t)t1.z;
    }
}

template <int DIM, int DK, bool PACKED>
__global__ void __launch_bounds__(256)
k_heis_compact(const DevModel m, float4* __restrict__ cs, const int4* __restrict__ tab,
               const int* __restrict__ fill_n, const float4* __restrict__ bh,
               const unsigned long long* __restrict__ sweep, const int* __restrict__ chains, int colour,
               unsigned sweep_off) {
    const int chain = chains[blockIdx.y];
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int seg = chain * 2 + colour;
    if (j >= fill_n[seg]) return;
    const size_t NH = (size_t)m.nhalf;
    int nbi[6];
    uint32_t box;
    compact_entry<PACKED>(tab, seg, NH, j, nbi, box);
    float4* own = cs + (size_t)seg * NH;
    const float4* oth = cs + (size_t)(chain * 2 + (colour ^ 1)) * NH;
    constexpr int ND = 2 * DIM;
    float nx[ND], ny[ND], nz[ND];
#pragma unroll
    for (int k = 0; k < ND; ++k) {   // one 16-byte load per neighbour (x, y, z, 0)
        const int q = nbi[k];
        const float4 v = q >= 0 ? __ldg(oth + q) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        nx[k] = v.x;
        ny[k] = v.y;
        nz[k] = v.z;
    }
    const float4 s = own[j];
    const float4 p = bh[chain];
    const nmmc_u4 r = sweep_draw(m, box, sweep[chain] + sweep_off, (uint32_t)chain);
    float tx, ty, tz;
    if (heis_attempt<ND, DK>(m, s.x, s.y, s.z, nx, ny, nz, p, r, tx, ty, tz)) own[j] = make_float4(tx, ty, tz, 0.0f);
}

// Filled sites' spins between the box planes and the compact planes of the listed chains
// (grid.y = 2 x chains: chain, colour). The compact planes hold one float4 (x, y, z, 0) per
// filled site, so that a neighbour is one 16-byte load.
__global__ void __launch_bounds__(256)
k_compact_copy(float4* __restrict__ cs, float* __restrict__ spins, const uint32_t* __restrict__ fill,
               const int* __restrict__ fill_n, const int* __restrict__ chains, int nhalf, size_t P,
               int to_compact) {
    const int chain = chains[blockIdx.y >> 1];
    const int seg = chain * 2 + (int)(blockIdx.y & 1);
    const int n = fill_n[seg];
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const size_t i = fill[(size_t)seg * nhalf + j];
        float* b = spins + (size_t)seg * 3 * P + i;
        float4* q = cs + (size_t)seg * nhalf + j;
        if (to_compact) {
            *q = make_float4(b[0], b[P], b[2 * P], 0.0f);
        } else {
            const float4 v = *q;
            b[0] = v.x;
            b[P] = v.y;
            b[2 * P] = v.z;
        }
    }
}

// Rows of SPT consecutive same-colour sites as one vector load: float4 (4 sites) or float2 (2).
template <int SPT> struct SiteVec { using T = float4; };
template <> struct SiteVec<2> { using T = float2; };
__device__ __forceinline__ float vel(const float4& v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w)); }
__device__ __forceinline__ float vel(const float2& v, int k) { return k == 0 ? v.x : v.y; }
__device__ __forceinline__ float4 make_vec(const float (&a)[4]) { return make_float4(a[0], a[1], a[2], a[3]); }
__device__ __forceinline__ float2 make_vec(const float (&a)[2]) { return make_float2(a[0], a[1]); }

// Block sums of NV per-thread FP32 values: FP32 warp sums, then FP64 across the block's warps
// on the lanes that own each value (every thread of the block must call it, from the same
// place); writes NV doubles.
template <int NV>
__device__ __forceinline__ void meas_block_rows(const float* acc, double* __restrict__ out) {
    __shared__ float red[NV][8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        float v = acc[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[k][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < NV) {
        double v = 0;
        const int nw = blockDim.x >> 5;
        for (int w = 0; w < nw; ++w) v += (double)red[threadIdx.x][w];
        out[threadIdx.x] = v;
    }
}

// Four consecutive same-colour sites of one row per thread (unmasked lattices whose rows hold
// a multiple of 4 sites per colour). Own spins, the same-row and the +-y / +-z neighbour rows
// of the other colour come in as float4 loads; the one x-neighbour that falls outside the
// quad is a scalar load. Each site keeps its own Philox counter and the same per-site
// arithmetic as k_heis_half, so both kernels produce the same chain. The Philox draw of site
// k+1 is issued before the field of site k is computed (its latency overlaps that work).
//
// One quad (row `row`, first compact site h0) of one chain; the row's x offset of this colour
// (x = 2h + xp) comes from (y + z + colour) per thread. With MEAS the quad's final spins are
// summed into macc (see k_heis_half_q4); `active` false computes without storing or summing.
template <int DIM, bool PERIODIC, int DK, int SPT, int MEAS>
__device__ __forceinline__ void q4_quad(const DevModel& m, float* __restrict__ spins, const float4* __restrict__ bh,
                                        const unsigned long long* __restrict__ sweep, unsigned sweep_off, int chain,
                                        int colour, int row, int h0, bool active, float* macc, float esign) {
    using VT = typename SiteVec<SPT>::T;
    int y, z;
    if (DIM == 3) {
        z = (m.ly_shift >= 0) ? (row >> m.ly_shift) : (row / m.ly);
        y = row - z * m.ly;
    } else {
        z = 0;
        y = row;
    }
    const int xp = (y + z + colour) & 1;   // x = 2h + xp
    const size_t P = (size_t)m.nhalf_pad;
    float* own = spins + ((size_t)chain * 2 + colour) * 3 * P;
    const float* oth = spins + ((size_t)chain * 2 + (colour ^ 1)) * 3 * P;
    const int rb = row * m.hx + h0;

    VT s[3], same[3], yp[3], ym[3], zp[3], zm[3];
    const VT vz = {};
    float ex[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        s[c] = *reinterpret_cast<const VT*>(own + c * P + rb);
        same[c] = __ldg(reinterpret_cast<const VT*>(oth + c * P + rb));
    }
    // x-neighbour outside the quad: h0-1 (xp = 0) or h0+4 (xp = 1)
    int hx_out = xp ? h0 + SPT : h0 - 1;
    bool ex_ok = true;
    if (PERIODIC) hx_out = (hx_out < 0) ? m.hx - 1 : (hx_out >= m.hx ? 0 : hx_out);
    else ex_ok = hx_out >= 0 && hx_out < m.hx;
#pragma unroll
    for (int c = 0; c < 3; ++c) ex[c] = ex_ok ? __ldg(oth + c * P + row * m.hx + hx_out) : 0.0f;
    // +-y rows
    {
        int yu = y + 1, yd = y - 1;
        bool okU = true, okD = true;
        if (PERIODIC) {
            yu = (yu == m.edge) ? 0 : yu;
            yd = (yd < 0) ? m.edge - 1 : yd;
        } else {
            okU = yu < m.edge;
            okD = yd >= 0;
        }
        const int ru = (z * m.ly + yu) * m.hx + h0, rd = (z * m.ly + yd) * m.hx + h0;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            yp[c] = okU ? __ldg(reinterpret_cast<const VT*>(oth + c * P + ru)) : vz;
            ym[c] = okD ? __ldg(reinterpret_cast<const VT*>(oth + c * P + rd)) : vz;
        }
    }
    if (DIM == 3) {
        int zu = z + 1, zd = z - 1;
        bool okU = true, okD = true;
        if (PERIODIC) {
            zu = (zu == m.edge) ? 0 : zu;
            zd = (zd < 0) ? m.edge - 1 : zd;
        } else {
            okU = zu < m.lz;
            okD = zd >= 0;
        }
        const int ru = (zu * m.ly + y) * m.hx + h0, rd = (zd * m.ly + y) * m.hx + h0;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            zp[c] = okU ? __ldg(reinterpret_cast<const VT*>(oth + c * P + ru)) : vz;
            zm[c] = okD ? __ldg(reinterpret_cast<const VT*>(oth + c * P + rd)) : vz;
        }
    }
    const float4 p = bh[chain];
    const unsigned long long sw = sweep[chain] + sweep_off;
    const uint32_t boxrow = (uint32_t)(m.edge * (y + m.edge * z));
    constexpr int ND = 2 * DIM;
    bool any = false;
    nmmc_u4 rnext = sweep_draw<true>(m, boxrow + (uint32_t)(2 * h0 + xp), sw, (uint32_t)chain);
    float out[3][SPT];
#pragma unroll
    for (int k = 0; k < SPT; ++k) {
        float nx[ND], ny[ND], nz[ND];
        float* nn[3] = {nx, ny, nz};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            // the neighbour of site h0+k at compact h0+k (same) and at h0+k-1 or h0+k+1 (shifted)
            float sm = vel(same[c], k);
            float sh = xp ? (k < SPT - 1 ? vel(same[c], k + 1) : ex[c]) : (k > 0 ? vel(same[c], k - 1) : ex[c]);
            float plusx = xp ? sh : sm, minusx = xp ? sm : sh;
            if (!PERIODIC) {
                // open x boundary: the site at x = edge-1 has no +x neighbour, x = 0 no -x
                const int x = 2 * (h0 + k) + xp;
                if (x + 1 >= m.edge) plusx = 0.0f;
                if (x == 0) minusx = 0.0f;
            }
            nn[c][0] = plusx;
            nn[c][1] = minusx;
            nn[c][2] = vel(yp[c], k);
            nn[c][3] = vel(ym[c], k);
            if (DIM == 3) {
                nn[c][4] = vel(zp[c], k);
                nn[c][5] = vel(zm[c], k);
            }
        }
        const float sx = vel(s[0], k), sy = vel(s[1], k), sz = vel(s[2], k);
        float tx, ty, tz;
        const nmmc_u4 r = rnext;
        if (k < SPT - 1) rnext = sweep_draw<true>(m, boxrow + (uint32_t)(2 * (h0 + k + 1) + xp), sw, (uint32_t)chain);
        float hx, hy, hz;
        heis_field<ND, DK>(m, nx, ny, nz, p, hx, hy, hz);
        const bool acc = heis_try(hx, hy, hz, sx, sy, sz, p, r, tx, ty, tz);
        out[0][k] = acc ? tx : sx;
        out[1][k] = acc ? ty : sy;
        out[2][k] = acc ? tz : sz;
        any |= acc;
        if (MEAS && active) {
            float dx, dy, dz;
            heis_dmi_part<ND, DK>(m, nx, ny, nz, dx, dy, dz);
            const float fx = fmaf(esign, dx, hx - p.y), fy = fmaf(esign, dy, hy - p.z), fz = fmaf(esign, dz, hz - p.w);
            macc[0] = fmaf(out[0][k], fx, fmaf(out[1][k], fy, fmaf(out[2][k], fz, macc[0])));
        }
    }
    if (any && active) {
#pragma unroll
        for (int c = 0; c < 3; ++c)
            *reinterpret_cast<VT*>(own + c * P + rb) = make_vec(out[c]);
    }
    if (MEAS && active) {
        // this quad's new colour-1 spins (M of colour 1); the colour-0 sites at the quad's
        // compact indices of the same row, final since the step's last colour-0 half-sweep
        // (every colour-0 site is in exactly one colour-1 quad's same-row vector): M of colour
        // 0, which is submag(0), and sub4mag, whose sites are all of colour 0
#pragma unroll
        for (int k = 0; k < SPT; ++k) {
            macc[1] += out[0][k];
            macc[2] += out[1][k];
            macc[3] += out[2][k];
            macc[4] += vel(same[0], k);
            macc[5] += vel(same[1], k);
            macc[6] += vel(same[2], k);
        }
        // sub4mag's sites (x+y, y-x+e4 and z all = 0 or all = 2 mod 4 with C's signed %,
        // e4 = edge - edge % 4) lie in the planes z = 0, 2 mod 4; x+y >= 0, and a negative
        // y-x+e4 can only match 0
        const int zz = (DIM == 3) ? (z & 3) : 0;
        if ((zz & 1) == 0) {
            const int e4 = m.edge - m.edge % 4;
#pragma unroll
            for (int k = 0; k < SPT; ++k) {
                const int x = 2 * (h0 + k) + (xp ^ 1);
                const int possum = x + y, posdiff = y - x + e4;
                if ((possum & 3) == zz && (posdiff & 3) == zz && (posdiff >= 0 || zz == 0)) {
                    macc[7] += vel(same[0], k);
                    macc[8] += vel(same[1], k);
                    macc[9] += vel(same[2], k);
                }
            }
        }
    }
}

// MEAS = 1 is the last colour-1 half-sweep of a sample step with the observables but the charge
// summed on the way (nmmc_sweep_measure on this path): every bond joins one site of each colour,
// and colour 0 is final after the step's last colour-0 half-sweep, colour 1 after this one. It
// sums s_i . h_E(i) over the bonds of each colour-1 site (h_E the energy's field,
// Old/lib/thermodynamics.cpp:71-96, which is h - H of the sweep plus esign times the sweep's DMI
// part: -2 with the reference's sign, 0 with the consistent one; tables whose +-axis records
// are pairs only), M of both colours (the colour-0 sum is submag(0), the sites with x+y+z even,
// :113-136) and the sub4mag sites (all of colour 0, :138-163), the colour-0 spins from the
// same-row vectors the update reads anyway. Each thread takes `qpt` quads (slots t, t + stride,
// ...), so that the block's sums cost little per site: FP32 per thread and per warp, FP64
// across the block's warps, one row of 10 doubles per block in mpart (2 e, M of colour 1, M of
// colour 0, sub4M).
//
// pf > 0 (plain launches): before its own work, each block asks L2 for the spins that block
// pf launches later in the grid (about one wave of resident blocks ahead) reads first: its own
// colour's rows and the other colour's same rows, 3 components each (192 lines of 128 B for
// 256 quads of 4 sites). By the time that block runs, its first loads hit L2 instead of
// waiting on DRAM; the prefetch changes no value.
template <int DIM, bool PERIODIC, int DK, int MINB, int SPT = 4, int MEAS = 0>
__global__ void __launch_bounds__(256, MINB)
k_heis_half_q4(const DevModel m, float* __restrict__ spins, const float4* __restrict__ bh,
               const unsigned long long* __restrict__ sweep, const int* __restrict__ chains,
               int colour, unsigned sweep_off, int qpt, double* __restrict__ mpart, float esign, int pf,
               int nchain_list) {
    const int chain = chains[blockIdx.y];
    const int qpr = m.hx / SPT;
    const int nquads = qpr * m.ly * m.lz;
    if (MEAS == 0 && pf > 0 && SPT == 4 && threadIdx.x < 192) {
        const long tgt = (long)blockIdx.y * gridDim.x + blockIdx.x + pf;
        const int ty = (int)(tgt / gridDim.x), tx = (int)(tgt - (long)ty * gridDim.x);
        const int q0 = tx * 256;
        if (ty < nchain_list && q0 < nquads) {
            const int sel = threadIdx.x / 96, c = (threadIdx.x % 96) >> 5, line = threadIdx.x & 31;
            const size_t P = (size_t)m.nhalf_pad;
            const int tch = chains[ty];
            const float* base = spins + (((size_t)tch * 2 + (colour ^ sel)) * 3 + c) * P + (size_t)q0 * SPT;
            const size_t end_off = (size_t)nquads * SPT;   // the plane's last site
            if ((size_t)q0 * SPT + (size_t)line * 32 < end_off)
                asm volatile("prefetch.global.L2 [%0];" ::"l"(base + (size_t)line * 32));
        }
    }
    const int qshift = (m.qpr_shift >= 0) ? m.qpr_shift + (SPT == 2 ? 1 : 0) : -1;   // log2(hx / SPT)
    constexpr int NV = MEAS ? 10 : 1;
    float macc[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) macc[v] = 0.0f;
    const int stride = gridDim.x * blockDim.x;
    const int nit = (MEAS == 0) ? 1 : qpt;
    for (int i = 0; i < nit; ++i) {
        const int t0 = blockIdx.x * blockDim.x + threadIdx.x + i * stride;
        // slots past the last quad: none in a plain launch; with MEAS every thread of the
        // block must reach the block reduction's barrier from the same place, so such a slot
        // works on the last quad and neither stores nor sums
        const bool active = t0 < nquads;
        if (MEAS == 0 && !active) return;
        const int q = active ? t0 : nquads - 1;
        const int row = (qshift >= 0) ? (q >> qshift) : (q / qpr);
        const int h0 = (q - row * qpr) * SPT;
        q4_quad<DIM, PERIODIC, DK, SPT, MEAS>(m, spins, bh, sweep, sweep_off, chain, colour, row, h0,
                                              MEAS == 0 || active, macc, esign);
    }
    if (MEAS != 0) {
        macc[0] *= 2.0f;   // the energy's pair sum counts every bond twice (exact)
        meas_block_rows<NV>(macc, mpart + ((size_t)blockIdx.y * gridDim.x + blockIdx.x) * NV);
    }
}

// ------------------------------------------------------------------------------------------
// Ring-pipelined 3-D half-sweep (periodic, unmasked, 64 sites per row and colour, i.e. edge
// 128): one CTA owns ROWS rows (y0 .. y0+ROWS-1) of one chain and colour over `zseg`
// consecutive z-planes and marches along z. The other colour's rows y0-1 .. y0+ROWS of each
// plane sit in a ring of NS shared-memory slots, the own colour's ROWS rows in two; every
// slot is filled by cp.async.bulk copies of contiguous row runs that complete on the slot's
// mbarrier (transaction bytes). Step z reads other-colour planes z-1, z, z+1 and own plane z;
// after the step's single CTA barrier, thread 0 refills the slot of plane z-1 with plane
// z-1+NS and the own slot of plane z with plane z+2, so with NS = 4 a copy is issued a whole
// step before the step that first needs it (NS = 3 would leave it none). The thread owns four
// consecutive same-colour sites of one row; their per-site arithmetic and Philox counters are
// those of k_heis_half_q4, so the chain is the same. Main-loop waits poll at most `limit`
// times; on a give-up the CTA sets *flag = 3, waits (bounded) for its copies in flight and
// exits, and nmmc_synchronize reports NMMC_ERR_TIMEOUT.
// ------------------------------------------------------------------------------------------
constexpr int kRingHx = 64;                                    // compact sites per row (edge 128)
constexpr unsigned kWaitLimit = 1u << 26;                      // default and drain poll bound

template <int ROWS, int NS>
struct RingShape {
    static constexpr int threads = ROWS * (kRingHx / 4);
    static constexpr int oth_slot = 3 * (ROWS + 2) * kRingHx;  // floats
    static constexpr int own_slot = 3 * ROWS * kRingHx;
    static constexpr size_t smem = (size_t)(NS * oth_slot + 2 * own_slot) * sizeof(float) +
                                   (NS + 2) * sizeof(unsigned long long);
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Waits for phase `parity` of `bar` with at most `limit` polls; false (and the error flag set)
// when they run out.
__device__ __forceinline__ bool ring_wait(unsigned long long* bar, unsigned parity, unsigned limit, int* flag) {
    for (unsigned it = 0; it < limit; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    atomicExch(flag, 3);
    return false;
}

// The four updates of one thread's quad from shared-memory rows: W own rows of this plane,
// O0 / Om / Op the other colour's rows (with one halo row each side) of planes z, z-1, z+1.
template <int DK, int ROWS>
__device__ __forceinline__ void ring_quad(const DevModel& m, float* __restrict__ gown, size_t P, const float* W,
                                          const float* O0, const float* Om, const float* Op, int r, int h0,
                                          int y, int z, int colour, float4 p, unsigned long long sw, int chain) {
    constexpr int ND = 6;
    auto el = [](const float4& v, int k) -> float { return k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w)); };
    const int E = m.edge;
    const int xp = (y + z + colour) & 1;
    float4 sv[3], same[3], yp[3], ym[3], zp[3], zm[3];
    float ex[3];
    const int hx_out = xp ? ((h0 + 4) & (kRingHx - 1)) : ((h0 - 1) & (kRingHx - 1));
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const int ob = c * (ROWS + 2) * kRingHx;
        sv[c] = *reinterpret_cast<const float4*>(W + c * ROWS * kRingHx + r * kRingHx + h0);
        same[c] = *reinterpret_cast<const float4*>(O0 + ob + (r + 1) * kRingHx + h0);
        yp[c] = *reinterpret_cast<const float4*>(O0 + ob + (r + 2) * kRingHx + h0);
        ym[c] = *reinterpret_cast<const float4*>(O0 + ob + r * kRingHx + h0);
        zp[c] = *reinterpret_cast<const float4*>(Op + ob + (r + 1) * kRingHx + h0);
        zm[c] = *reinterpret_cast<const float4*>(Om + ob + (r + 1) * kRingHx + h0);
        ex[c] = O0[ob + (r + 1) * kRingHx + hx_out];
    }
    const uint32_t boxrow = (uint32_t)(E * (y + E * z));
    bool any = false;
    float out[3][4];
    nmmc_u4 rnext = sweep_draw<true>(m, boxrow + (uint32_t)(2 * h0 + xp), sw, (uint32_t)chain);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        float nx[ND], ny[ND], nz[ND];
        float* nn[3] = {nx, ny, nz};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float smv = el(same[c], k);
            const float sh = xp ? (k < 3 ? el(same[c], k + 1) : ex[c]) : (k > 0 ? el(same[c], k - 1) : ex[c]);
            nn[c][0] = xp ? sh : smv;
            nn[c][1] = xp ? smv : sh;
            nn[c][2] = el(yp[c], k);
            nn[c][3] = el(ym[c], k);
            nn[c][4] = el(zp[c], k);
            nn[c][5] = el(zm[c], k);
        }
        const float sx = el(sv[0], k), sy = el(sv[1], k), sz = el(sv[2], k);
        const nmmc_u4 rr = rnext;
        if (k < 3) rnext = sweep_draw<true>(m, boxrow + (uint32_t)(2 * (h0 + k + 1) + xp), sw, (uint32_t)chain);
        float hx, hy, hz, tx, ty, tz;
        heis_field<ND, DK>(m, nx, ny, nz, p, hx, hy, hz);
        const bool acc = heis_try(hx, hy, hz, sx, sy, sz, p, rr, tx, ty, tz);
        out[0][k] = acc ? tx : sx;
        out[1][k] = acc ? ty : sy;
        out[2][k] = acc ? tz : sz;
        any |= acc;
    }
    if (any) {
        const size_t gb = ((size_t)z * m.ly + y) * kRingHx + h0;
#pragma unroll
        for (int c = 0; c < 3; ++c)
            *reinterpret_cast<float4*>(gown + c * P + gb) = make_float4(out[c][0], out[c][1], out[c][2], out[c][3]);
    }
}

template <int DK, int ROWS, int NS, int MINB>
__global__ void __launch_bounds__(RingShape<ROWS, NS>::threads, MINB)
k_heis_half_ring(const DevModel m, float* __restrict__ spins, const float4* __restrict__ bh,
                 const unsigned long long* __restrict__ sweep, const int* __restrict__ chains, int colour,
                 unsigned sweep_off, int zseg, unsigned limit, int* __restrict__ flag) {
    using RS = RingShape<ROWS, NS>;
    extern __shared__ __align__(128) float psm[];
    float* oth = psm;                                   // NS slots of [3][ROWS + 2][64]
    float* ownb = psm + NS * RS::oth_slot;              // 2 slots of [3][ROWS][64]
    unsigned long long* bar = reinterpret_cast<unsigned long long*>(ownb + 2 * RS::own_slot);   // NS + 2
    const int chain = chains[blockIdx.y];
    const int ntile = m.ly / ROWS;
    const int ytile = blockIdx.x % ntile, zs = blockIdx.x / ntile;
    const int y0 = ytile * ROWS, z0 = zs * zseg, z1 = min(z0 + zseg, m.lz);
    const size_t P = (size_t)m.nhalf_pad;
    float* gown = spins + ((size_t)chain * 2 + colour) * 3 * P;
    const float* goth = spins + ((size_t)chain * 2 + (colour ^ 1)) * 3 * P;
    const int E = m.edge;
    const unsigned rowb = kRingHx * sizeof(float);

    if (threadIdx.x == 0) {
        for (int i = 0; i < NS + 2; ++i) mbar_init(&bar[i], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    // plane zp (z0-1 <= zp <= z1) is fill (zp - z0 + 1) / NS of other-colour slot
    // (zp - z0 + 1) % NS, and own plane zp fill (zp - z0) / 2 of own slot (zp - z0) % 2; a fill
    // completes the barrier phase of its parity
    auto oslot = [&](int zp) { return (zp - z0 + 1) % NS; };
    auto opar = [&](int zp) { return (unsigned)(((zp - z0 + 1) / NS) & 1); };
    auto wpar = [&](int zp) { return (unsigned)(((zp - z0) >> 1) & 1); };
    // producer (thread 0): rows y0-1 .. y0+ROWS of other-colour plane zp (periodic), split
    // where they wrap; ROWS own-colour rows of plane zp
    auto load_oth = [&](int zp) {
        const int zz = (zp + E) % E;
        const int slot = oslot(zp);
        float* dst = oth + slot * RS::oth_slot;
        mbar_expect_tx(&bar[slot], 3u * (ROWS + 2) * rowb);
        for (int c = 0; c < 3; ++c) {
            const float* src = goth + c * P + (size_t)zz * m.ly * kRingHx;
            float* d = dst + c * (ROWS + 2) * kRingHx;
            int r = 0;
            while (r < ROWS + 2) {
                const int y = (y0 - 1 + r + E) % E;
                const int run = min(ROWS + 2 - r, E - y);
                bulk_g2s(d + r * kRingHx, src + (size_t)y * kRingHx, (unsigned)run * rowb, &bar[slot]);
                r += run;
            }
        }
    };
    auto load_own = [&](int zp) {
        const int slot = (zp - z0) & 1;
        float* dst = ownb + slot * RS::own_slot;
        mbar_expect_tx(&bar[NS + slot], 3u * ROWS * rowb);
        for (int c = 0; c < 3; ++c)
            bulk_g2s(dst + c * ROWS * kRingHx, gown + c * P + ((size_t)zp * m.ly + y0) * kRingHx,
                     (unsigned)ROWS * rowb, &bar[NS + slot]);
    };
    if (threadIdx.x == 0) {
        for (int zp = z0 - 1; zp <= min(z0 + NS - 2, z1); ++zp) load_oth(zp);
        load_own(z0);
        if (z0 + 1 < z1) load_own(z0 + 1);
    }
    constexpr int TPR = kRingHx / 4;
    const int r = threadIdx.x / TPR, h0 = (threadIdx.x % TPR) * 4;
    const int y = y0 + r;
    const float4 p = bh[chain];
    const unsigned long long sw = sweep[chain] + sweep_off;
    int z = z0;
    for (; z < z1; ++z) {
        const int sm1 = oslot(z - 1), s0 = oslot(z), sp1 = oslot(z + 1);
        const int so = (z - z0) & 1;
        bool ok = true;
        if (z == z0) ok = ring_wait(&bar[sm1], opar(z - 1), limit, flag) && ring_wait(&bar[s0], opar(z), limit, flag);
        ok = ok && ring_wait(&bar[sp1], opar(z + 1), limit, flag);
        ok = ok && ring_wait(&bar[NS + so], wpar(z), limit, flag);
        if (ok)
            ring_quad<DK, ROWS>(m, gown, P, ownb + so * RS::own_slot, oth + s0 * RS::oth_slot,
                                oth + sm1 * RS::oth_slot, oth + sp1 * RS::oth_slot, r, h0, y, z, colour, p, sw,
                                chain);
        // one barrier per step: the slots of other plane z-1 and own plane z are free
        // afterwards; all threads leave together if any wait gave up
        if (__syncthreads_or(!ok)) break;
        if (threadIdx.x == 0) {
            fence_proxy_async();
            if (z - 1 + NS <= z1) load_oth(z - 1 + NS);
            if (z + 2 < z1) load_own(z + 2);
        }
    }
    // After a give-up the loop stopped at the barrier of step z, before that step's refills:
    // the other-colour planes issued are z0-1 .. min(z+NS-2, z1) and the own planes z0 ..
    // min(z+1, z1-1), one fill per slot possibly still landing. Give each slot's last fill a
    // bounded time to complete before the CTA's shared memory is released.
    if (z < z1 && threadIdx.x == 0) {
        const int ho = min(z + NS - 2, z1), hw = min(z + 1, z1 - 1);
        for (int zp = max(z0 - 1, ho - NS + 1); zp <= ho; ++zp)
            for (unsigned it = 0; it < (kWaitLimit >> 4); ++it)
                if (mbar_try_wait(&bar[oslot(zp)], opar(zp))) break;
        for (int zp = max(z0, hw - 1); zp <= hw; ++zp)
            for (unsigned it = 0; it < (kWaitLimit >> 4); ++it)
                if (mbar_try_wait(&bar[NS + ((zp - z0) & 1)], wpar(zp))) break;
    }
}

// Warp-specialised form of the ring kernel: warp 0 is the producer (its lane 0 issues every
// bulk copy), the other ROWS/2 warps consume. There is no CTA-wide barrier per step: each
// consumer warp releases other-colour plane z-1 and own plane z after reading its step z
// data by arriving on the slot's "empty" mbarrier (one arrival per consumer warp), and the
// producer waits for that release before it refills the slot. The consumer warps may drift
// apart by up to the ring's slack. Every wait is bounded by `limit` polls and also ends when
// another warp of the CTA gave up (a shared abort word); the producer then lets every copy it
// issued land before the CTA exits. Same per-site arithmetic and Philox counters as
// k_heis_half_q4.
template <int ROWS, int NS>
struct WsShape {
    static constexpr int consumers = ROWS * (kRingHx / 4);
    static constexpr int threads = consumers + 32;
    static constexpr int oth_slot = 3 * (ROWS + 2) * kRingHx;
    static constexpr int own_slot = 3 * ROWS * kRingHx;
    static constexpr size_t smem = (size_t)(NS * oth_slot + 2 * own_slot) * sizeof(float) +
                                   2 * (NS + 2) * sizeof(unsigned long long) + 16;
};

__device__ __forceinline__ void mbar_arrive(unsigned long long* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool ws_wait(unsigned long long* bar, unsigned parity, unsigned limit, int* flag,
                                        volatile int* abort) {
    for (unsigned it = 0; it < limit; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if (*abort) return false;
    }
    *abort = 1;
    atomicExch(flag, 3);
    return false;
}

template <int DK, int ROWS, int NS, int MINB>
__global__ void __launch_bounds__(WsShape<ROWS, NS>::threads, MINB)
k_heis_half_ws(const DevModel m, float* __restrict__ spins, const float4* __restrict__ bh,
               const unsigned long long* __restrict__ sweep, const int* __restrict__ chains, int colour,
               unsigned sweep_off, int zseg, unsigned limit, int* __restrict__ flag) {
    using WS = WsShape<ROWS, NS>;
    constexpr int NCW = WS::consumers / 32;
    extern __shared__ __align__(128) float psm[];
    float* oth = psm;                                   // NS slots of [3][ROWS + 2][64]
    float* ownb = psm + NS * WS::oth_slot;              // 2 slots of [3][ROWS][64]
    unsigned long long* full = reinterpret_cast<unsigned long long*>(ownb + 2 * WS::own_slot);   // NS + 2
    unsigned long long* empty = full + (NS + 2);                                                // NS + 2
    volatile int* abort = reinterpret_cast<volatile int*>(empty + (NS + 2));
    const int chain = chains[blockIdx.y];
    const int ntile = m.ly / ROWS;
    const int ytile = blockIdx.x % ntile, zs = blockIdx.x / ntile;
    const int y0 = ytile * ROWS, z0 = zs * zseg, z1 = min(z0 + zseg, m.lz);
    const size_t P = (size_t)m.nhalf_pad;
    float* gown = spins + ((size_t)chain * 2 + colour) * 3 * P;
    const float* goth = spins + ((size_t)chain * 2 + (colour ^ 1)) * 3 * P;
    const int E = m.edge;
    const unsigned rowb = kRingHx * sizeof(float);

    if (threadIdx.x == 0) {
        for (int i = 0; i < NS + 2; ++i) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], NCW);
        }
        *abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    auto oslot = [&](int zp) { return (zp - z0 + 1) % NS; };
    auto opar = [&](int zp) { return (unsigned)(((zp - z0 + 1) / NS) & 1); };
    auto wpar = [&](int zp) { return (unsigned)(((zp - z0) >> 1) & 1); };
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == 0) {
        if (lane != 0) return;
        auto load_oth = [&](int zp) {
            const int zz = (zp + E) % E;
            const int slot = oslot(zp);
            float* dst = oth + slot * WS::oth_slot;
            mbar_expect_tx(&full[slot], 3u * (ROWS + 2) * rowb);
            for (int c = 0; c < 3; ++c) {
                const float* src = goth + c * P + (size_t)zz * m.ly * kRingHx;
                float* d = dst + c * (ROWS + 2) * kRingHx;
                int r = 0;
                while (r < ROWS + 2) {
                    const int y = (y0 - 1 + r + E) % E;
                    const int run = min(ROWS + 2 - r, E - y);
                    bulk_g2s(d + r * kRingHx, src + (size_t)y * kRingHx, (unsigned)run * rowb, &full[slot]);
                    r += run;
                }
            }
        };
        auto load_own = [&](int zp) {
            const int slot = (zp - z0) & 1;
            float* dst = ownb + slot * WS::own_slot;
            mbar_expect_tx(&full[NS + slot], 3u * ROWS * rowb);
            for (int c = 0; c < 3; ++c)
                bulk_g2s(dst + c * ROWS * kRingHx, gown + c * P + ((size_t)zp * m.ly + y0) * kRingHx,
                         (unsigned)ROWS * rowb, &full[NS + slot]);
        };
        int ho = z0 - 2, hw = z0 - 1;   // last other / own plane issued
        for (int zp = z0 - 1; zp <= min(z0 + NS - 2, z1); ++zp) {
            load_oth(zp);
            ho = zp;
        }
        load_own(z0);
        hw = z0;
        if (z0 + 1 < z1) {
            load_own(z0 + 1);
            hw = z0 + 1;
        }
        for (int z = z0; z < z1; ++z) {
            // every consumer warp has read its step z: other plane z-1 and own plane z are free
            if (z - 1 + NS <= z1) {
                if (!ws_wait(&empty[oslot(z - 1)], opar(z - 1), limit, flag, abort)) break;
                fence_proxy_async();
                load_oth(z - 1 + NS);
                ho = z - 1 + NS;
            }
            if (z + 2 < z1) {
                if (!ws_wait(&empty[NS + ((z - z0) & 1)], wpar(z), limit, flag, abort)) break;
                fence_proxy_async();
                load_own(z + 2);
                hw = z + 2;
            }
        }
        // the last fill of every slot lands before the CTA's shared memory can be released
        for (int zp = max(z0 - 1, ho - NS + 1); zp <= ho; ++zp)
            for (unsigned it = 0; it < (kWaitLimit >> 4); ++it)
                if (mbar_try_wait(&full[oslot(zp)], opar(zp))) break;
        for (int zp = max(z0, hw - 1); zp <= hw; ++zp)
            for (unsigned it = 0; it < (kWaitLimit >> 4); ++it)
                if (mbar_try_wait(&full[NS + ((zp - z0) & 1)], wpar(zp))) break;
        return;
    }
    constexpr int TPR = kRingHx / 4;
    const int ct = threadIdx.x - 32;
    const int r = ct / TPR, h0 = (ct % TPR) * 4;
    const int y = y0 + r;
    const float4 p = bh[chain];
    const unsigned long long sw = sweep[chain] + sweep_off;
    constexpr int ND = 6;
    auto el = [](const float4& v, int k) -> float { return k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w)); };
    for (int z = z0; z < z1; ++z) {
        const int sm1 = oslot(z - 1), s0 = oslot(z), sp1 = oslot(z + 1);
        const int so = (z - z0) & 1;
        bool ok = true;
        if (z == z0) ok = ws_wait(&full[sm1], opar(z - 1), limit, flag, abort) &&
                          ws_wait(&full[s0], opar(z), limit, flag, abort);
        ok = ok && ws_wait(&full[sp1], opar(z + 1), limit, flag, abort);
        ok = ok && ws_wait(&full[NS + so], wpar(z), limit, flag, abort);
        if (!ok) break;
        const float* O0 = oth + s0 * WS::oth_slot;
        const float* Om = oth + sm1 * WS::oth_slot;
        const float* Op = oth + sp1 * WS::oth_slot;
        const float* W = ownb + so * WS::own_slot;
        const int xp = (y + z + colour) & 1;
        float4 sv[3], same[3], yp[3], ym[3], zp[3], zm[3];
        float ex[3];
        const int hx_out = xp ? ((h0 + 4) & (kRingHx - 1)) : ((h0 - 1) & (kRingHx - 1));
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const int ob = c * (ROWS + 2) * kRingHx;
            sv[c] = *reinterpret_cast<const float4*>(W + c * ROWS * kRingHx + r * kRingHx + h0);
            same[c] = *reinterpret_cast<const float4*>(O0 + ob + (r + 1) * kRingHx + h0);
            yp[c] = *reinterpret_cast<const float4*>(O0 + ob + (r + 2) * kRingHx + h0);
            ym[c] = *reinterpret_cast<const float4*>(O0 + ob + r * kRingHx + h0);
            zp[c] = *reinterpret_cast<const float4*>(Op + ob + (r + 1) * kRingHx + h0);
            zm[c] = *reinterpret_cast<const float4*>(Om + ob + (r + 1) * kRingHx + h0);
            ex[c] = O0[ob + (r + 1) * kRingHx + hx_out];
        }
        // the warp's reads of other plane z-1 and own plane z are done: release them
        __syncwarp();
        if (lane == 0) {
            mbar_arrive(&empty[sm1]);
            mbar_arrive(&empty[NS + so]);
        }
        const uint32_t boxrow = (uint32_t)(E * (y + E * z));
        bool any = false;
        float out[3][4];
        nmmc_u4 rnext = sweep_draw<true>(m, boxrow + (uint32_t)(2 * h0 + xp), sw, (uint32_t)chain);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            float nx[ND], ny[ND], nz[ND];
            float* nn[3] = {nx, ny, nz};
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float smv = el(same[c], k);
                const float sh = xp ? (k < 3 ? el(same[c], k + 1) : ex[c]) : (k > 0 ? el(same[c], k - 1) : ex[c]);
                nn[c][0] = xp ? sh : smv;
                nn[c][1] = xp ? smv : sh;
                nn[c][2] = el(yp[c], k);
                nn[c][3] = el(ym[c], k);
                nn[c][4] = el(zp[c], k);
                nn[c][5] = el(zm[c], k);
            }
            const float sx = el(sv[0], k), sy = el(sv[1], k), sz = el(sv[2], k);
            const nmmc_u4 rr = rnext;
            if (k < 3) rnext = sweep_draw<true>(m, boxrow + (uint32_t)(2 * (h0 + k + 1) + xp), sw, (uint32_t)chain);
            float hx, hy, hz, tx, ty, tz;
            heis_field<ND, DK>(m, nx, ny, nz, p, hx, hy, hz);
            const bool acc = heis_try(hx, hy, hz, sx, sy, sz, p, rr, tx, ty, tz);
            out[0][k] = acc ? tx : sx;
            out[1][k] = acc ? ty : sy;
            out[2][k] = acc ? tz : sz;
            any |= acc;
        }
        if (any) {
            const size_t gb = ((size_t)z * m.ly + y) * kRingHx + h0;
#pragma unroll
            for (int c = 0; c < 3; ++c)
                *reinterpret_cast<float4*>(gown + c * P + gb) = make_float4(out[c][0], out[c][1], out[c][2], out[c][3]);
        }
    }
}

__global__ void k_advance(unsigned long long* sweep, const int* chains, int n, int nsweeps) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) sweep[chains[i]] += (unsigned long long)nsweeps;
}

template <int DIM, bool PERIODIC, bool MASKED, int DK>
static void heis_launch(Ctx& c, const int* d_chains, int n, int colour, unsigned off) {
    dim3 grid(((MASKED ? c.fill_max : c.m.nhalf) + 255) / 256, n);
    if (grid.x == 0) return;   // no filled site in any chain
    k_heis_half<DIM, PERIODIC, MASKED, DK><<<grid, 256, 0, c.stream>>>(
        c.m, (float*)c.d_spins, c.d_fill, c.d_fill_n, c.d_bh, c.d_sweep, d_chains, colour, off);
}

using HalfFn = void (*)(Ctx&, const int*, int, int, unsigned);

// Blocks of one chain in a four-site half-sweep launch; the fused measurement's launches give
// each thread kMeasQpt quads (their block count is the rows of mpart per chain).
constexpr int kMeasQpt = 4;
static int q4_blocks(const Ctx& c) { return ((c.m.hx >> 2) * c.m.ly * c.m.lz + 255) / 256; }
static int q4_meas_blocks(const Ctx& c) { return (q4_blocks(c) + kMeasQpt - 1) / kMeasQpt; }

template <int DIM, bool PERIODIC, int DK>
static void heis_q4_launch(Ctx& c, const int* d_chains, int n, int colour, unsigned off) {
    float* sp = (float*)c.d_spins;
    dim3 grid(q4_blocks(c), n);
    const int per_sm = c.half_kernel == 2 ? 2 : 3;
    // L2 prefetch distance in blocks: the option's waves of resident blocks ahead (0: off)
    const int pf = c.l2_prefetch > 0 ? c.l2_prefetch * c.sm_count * per_sm / 4 : 0;
    if (c.half_kernel == 2)   // register cap for 2 CTAs/SM (no spills)
        k_heis_half_q4<DIM, PERIODIC, DK, 2><<<grid, 256, 0, c.stream>>>(
            c.m, sp, c.d_bh, c.d_sweep, d_chains, colour, off, 1, nullptr, 0.0f, pf, n);
    else                      // 3 CTAs/SM (80 registers, more warps in flight)
        k_heis_half_q4<DIM, PERIODIC, DK, 3><<<grid, 256, 0, c.stream>>>(
            c.m, sp, c.d_bh, c.d_sweep, d_chains, colour, off, 1, nullptr, 0.0f, pf, n);
}

// The step's last colour-1 half-sweep with the observables but the charge summed on the way
// (rows of 10 doubles; see k_heis_half_q4).
template <int DIM, bool PERIODIC, int DK>
static void heis_q4_meas_launch(Ctx& c, const int* d_chains, int n, int colour, unsigned off) {
    float* sp = (float*)c.d_spins;
    const int nb = q4_meas_blocks(c);
    dim3 grid(nb, n);
    const float esign = c.dmi_sign ? 0.0f : -2.0f;
    k_heis_half_q4<DIM, PERIODIC, DK, 2, 4, 1><<<grid, 256, 0, c.stream>>>(
        c.m, sp, c.d_bh, c.d_sweep, d_chains, colour, off, kMeasQpt, c.d_mrows, esign, 0, n);
}

template <int DIM, bool PER>
static HalfFn pick_heis_q4_meas(int dk) {
    switch (dk) {
        case kDmiNone: return heis_q4_meas_launch<DIM, PER, kDmiNone>;
        case kDmiPairs: return heis_q4_meas_launch<DIM, PER, kDmiPairs>;
        default: return heis_q4_meas_launch<DIM, PER, kDmiAxial>;
    }
}


// z-planes per CTA of the ring kernels: the option's value, else the largest of 32 and 16 that
// gives at least eight CTAs per resident slot (the launch's last wave idles fewer SMs), else 8.
static int ring_zseg(const Ctx& c, int n, int rows, int per_sm) {
    if (c.ring_zseg > 0) return c.ring_zseg;
    const long slots = (long)c.sm_count * per_sm;
    for (int zs : {32, 16})
        if ((long)n * (c.m.ly / rows) * ((c.m.lz + zs - 1) / zs) >= 8 * slots) return zs;
    return 8;
}

template <int DK, int ROWS, int NS, int MINB>
static void heis_ring_launch_v(Ctx& c, const int* d_chains, int n, int colour, unsigned off) {
    using RS = RingShape<ROWS, NS>;
    auto kern = k_heis_half_ring<DK, ROWS, NS, MINB>;
    const uint32_t bit = 1u << ((DK * 4 + (ROWS == 8 ? 0 : 1) * 2 + (NS == 5 ? 1 : 0)) & 31);
    if (!(c.pipe_attr & bit)) {   // attribute set once on this context's device
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)RS::smem);
        c.pipe_attr |= bit;
    }
    const int zs = ring_zseg(c, n, ROWS, MINB);
    const int nblk = (c.m.ly / ROWS) * ((c.m.lz + zs - 1) / zs);
    dim3 grid(nblk, n);
    kern<<<grid, RS::threads, RS::smem, c.stream>>>(c.m, (float*)c.d_spins, c.d_bh, c.d_sweep, d_chains, colour,
                                                    off, zs, c.wait_limit, c.d_flag);
}

template <int DK, int ROWS, int NS, int MINB>
static void heis_ws_launch_v(Ctx& c, const int* d_chains, int n, int colour, unsigned off) {
    using WS = WsShape<ROWS, NS>;
    auto kern = k_heis_half_ws<DK, ROWS, NS, MINB>;
    const uint32_t bit = 1u << ((16 + DK * 4 + (NS == 5 ? 1 : 0)) & 31);
    if (!(c.pipe_attr & bit)) {   // attribute set once on this context's device
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)WS::smem);
        c.pipe_attr |= bit;
    }
    const int zs = ring_zseg(c, n, ROWS, MINB);
    const int nblk = (c.m.ly / ROWS) * ((c.m.lz + zs - 1) / zs);
    dim3 grid(nblk, n);
    kern<<<grid, WS::threads, WS::smem, c.stream>>>(c.m, (float*)c.d_spins, c.d_bh, c.d_sweep, d_chains, colour,
                                                    off, zs, c.wait_limit, c.d_flag);
}

// option 3: 8 rows, ring of 4 (5 CTAs/SM); 4: 16 rows, ring of 4 (2 CTAs/SM); 5: 8 rows, ring
// of 5 (4 CTAs/SM); 6 and 7: the warp-specialised form, 8 rows and a ring of 4 or 5 (4 CTAs/SM:
// at 5 the register cap of 160-thread CTAs spills)
template <int DK>
static void heis_ring_launch(Ctx& c, const int* d_chains, int n, int colour, unsigned off) {
    if (c.half_kernel == 6) heis_ws_launch_v<DK, 8, 4, 4>(c, d_chains, n, colour, off);
    else if (c.half_kernel == 7) heis_ws_launch_v<DK, 8, 5, 4>(c, d_chains, n, colour, off);
    else if (c.half_kernel == 4) heis_ring_launch_v<DK, 16, 4, 2>(c, d_chains, n, colour, off);
    else if (c.half_kernel == 5) heis_ring_launch_v<DK, 8, 5, 4>(c, d_chains, n, colour, off);
    else heis_ring_launch_v<DK, 8, 4, 5>(c, d_chains, n, colour, off);
}

static HalfFn pick_heis_ring(int dk) {
    switch (dk) {
        case kDmiNone: return heis_ring_launch<kDmiNone>;
        case kDmiGeneral: return heis_ring_launch<kDmiGeneral>;
        case kDmiPairs: return heis_ring_launch<kDmiPairs>;
        default: return heis_ring_launch<kDmiAxial>;
    }
}

// Lattices the ring kernels cover: 3-D periodic unmasked Heisenberg of edge 128.
static bool ring_fits(const Ctx& c) {
    return !c.ising && !c.masked && c.periodic && c.dim == 3 && c.m.hx == kRingHx && (c.m.ly % 16) == 0 &&
           !c.m.general;
}

template <int DIM, bool PERIODIC, bool MASKED>
static void ising_launch(Ctx& c, const int* d_chains, int n, int colour, unsigned off) {
    dim3 grid(((MASKED ? c.fill_max : c.m.nhalf) + 255) / 256, n);
    if (grid.x == 0) return;   // no filled site in any chain
    k_ising_half<DIM, PERIODIC, MASKED><<<grid, 256, 0, c.stream>>>(
        c.m, (int8_t*)c.d_spins, c.d_fill, c.d_fill_n, c.d_bh, c.d_sweep, d_chains, colour, off);
}

template <int DIM, bool PER, bool MSK>
static HalfFn pick_heis(int dk) {
    switch (dk) {
        case kDmiNone: return heis_launch<DIM, PER, MSK, kDmiNone>;
        case kDmiGeneral: return heis_launch<DIM, PER, MSK, kDmiGeneral>;
        case kDmiPairs: return heis_launch<DIM, PER, MSK, kDmiPairs>;
        default: return heis_launch<DIM, PER, MSK, kDmiAxial>;
    }
}

template <int DIM, bool PER>
static HalfFn pick_heis_q4(int dk) {
    switch (dk) {
        case kDmiNone: return heis_q4_launch<DIM, PER, kDmiNone>;
        case kDmiGeneral: return heis_q4_launch<DIM, PER, kDmiGeneral>;
        case kDmiPairs: return heis_q4_launch<DIM, PER, kDmiPairs>;
        default: return heis_q4_launch<DIM, PER, kDmiAxial>;
    }
}

static HalfFn pick_half(const Ctx& c) {
    const bool per = c.periodic, msk = c.masked;
    const int dk = c.m.dmi_kind;
    if (ring_fits(c) && c.half_kernel >= 3) return pick_heis_ring(dk);
    if (!c.ising && !msk && (c.m.hx % 4) == 0 && c.half_kernel != 1) {
        if (c.dim == 3) return per ? pick_heis_q4<3, true>(dk) : pick_heis_q4<3, false>(dk);
        return per ? pick_heis_q4<2, true>(dk) : pick_heis_q4<2, false>(dk);
    }
    if (c.ising) {
        if (c.dim == 3) {
            if (per) return msk ? ising_launch<3, true, true> : ising_launch<3, true, false>;
            return msk ? ising_launch<3, false, true> : ising_launch<3, false, false>;
        }
        if (per) return msk ? ising_launch<2, true, true> : ising_launch<2, true, false>;
        return msk ? ising_launch<2, false, true> : ising_launch<2, false, false>;
    }
    if (c.dim == 3) {
        if (per) return msk ? pick_heis<3, true, true>(dk) : pick_heis<3, true, false>(dk);
        return msk ? pick_heis<3, false, true>(dk) : pick_heis<3, false, false>(dk);
    }
    if (per) return msk ? pick_heis<2, true, true>(dk) : pick_heis<2, true, false>(dk);
    return msk ? pick_heis<2, false, true>(dk) : pick_heis<2, false, false>(dk);
}

int launch_advance(Ctx& c, const int* d_chains, int n, int nsweeps) {
    k_advance<<<(n + 127) / 128, 128, 0, c.stream>>>(c.d_sweep, d_chains, n, nsweeps);
    return cuda_check(cudaGetLastError(), "k_advance");
}

static bool use_compact(const Ctx& c) {
    return c.masked && !c.ising && !c.m.general && c.masked_compact == 0 && c.d_fill;
}

template <int DIM, int DK>
static void heis_compact_launch(Ctx& c, const int* d_chains, int n, int colour, unsigned off) {
    dim3 grid((c.fill_max + 255) / 256, n);
    if (grid.x == 0) return;
    if (c.ctab_packed)
        k_heis_compact<DIM, DK, true><<<grid, 256, 0, c.stream>>>(c.m, c.d_cspins, c.d_ctab, c.d_fill_n, c.d_bh,
                                                                   c.d_sweep, d_chains, colour, off);
    else
        k_heis_compact<DIM, DK, false><<<grid, 256, 0, c.stream>>>(c.m, c.d_cspins, c.d_ctab, c.d_fill_n, c.d_bh,
                                                                    c.d_sweep, d_chains, colour, off);
}

template <int DIM>
static HalfFn pick_compact(int dk) {
    switch (dk) {
        case kDmiNone: return heis_compact_launch<DIM, kDmiNone>;
        case kDmiGeneral: return heis_compact_launch<DIM, kDmiGeneral>;
        case kDmiPairs: return heis_compact_launch<DIM, kDmiPairs>;
        default: return heis_compact_launch<DIM, kDmiAxial>;
    }
}

static int compact_copy(Ctx& c, const int* d_chains, int n, bool to_compact) {
    if (c.fill_max == 0) return NMMC_OK;
    const int bx = std::min((c.fill_max + 255) / 256, 64);
    for (int c0 = 0; c0 < n; c0 += 32767) {   // grid.y = 2 x chains of this part
        const int part = std::min(32767, n - c0);
        k_compact_copy<<<dim3(bx, 2 * part), 256, 0, c.stream>>>(c.d_cspins, (float*)c.d_spins, c.d_fill, c.d_fill_n,
                                                                 d_chains + c0, c.m.nhalf, (size_t)c.m.nhalf_pad,
                                                                 to_compact ? 1 : 0);
    }
    return cuda_check(cudaGetLastError(), "k_compact_copy");
}

// One chain's table of the compact form, from its host mask (the same site order as its
// filled-site lists: z, y, x), in the context's format. Returns kTableDoesNotFit (nothing
// uploaded) when the packed format is in use and a neighbour difference does not fit in 16
// bits.
int compact_table_chain(Ctx& c, int chain) {
    const int E = c.edge, nz = c.m.lz, ND = 2 * c.dim;
    const size_t NH = (size_t)c.m.nhalf;
    const uint8_t* mk = &c.mask[(size_t)chain * c.box_sites];
    std::vector<int> pos((size_t)c.box_sites, -1);
    int cnt[2] = {0, 0};
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < E; ++y)
            for (int x = 0; x < E; ++x) {
                const long box = x + (long)E * (y + (long)E * z);
                if (mk[box]) pos[box] = cnt[(x + y + z) & 1]++;
            }
    if ((size_t)cnt[0] > NH || (size_t)cnt[1] > NH)
        return set_error(NMMC_ERR_ARG, "filled-site list longer than a colour plane");
    const int per = c.ctab_packed ? 1 : 2;
    std::vector<int4> tab[2];
    tab[0].resize((size_t)per * cnt[0]);
    tab[1].resize((size_t)per * cnt[1]);
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < E; ++y)
            for (int x = 0; x < E; ++x) {
                const long box = x + (long)E * (y + (long)E * z);
                if (!mk[box]) continue;
                const int colour = (x + y + z) & 1, j = pos[box];
                int nb[6] = {-1, -1, -1, -1, -1, -1};
                for (int k = 0; k < ND; ++k) {   // stencil order +x, -x, +y, -y, +z, -z (nb_compact)
                    int q[3] = {x + (k == 0) - (k == 1), y + (k == 2) - (k == 3), z + (k == 4) - (k == 5)};
                    bool ok = true;
                    for (int a = 0; a < c.dim; ++a) {
                        if (c.periodic) q[a] = (q[a] + E) % E;
                        else if (q[a] < 0 || q[a] >= E) ok = false;
                    }
                    if (ok) nb[k] = pos[q[0] + (long)E * (q[1] + (long)E * q[2])];
                }
                if (c.ctab_packed) {
                    uint32_t h[6];
                    for (int k = 0; k < 6; ++k) {
                        const int d = nb[k] < 0 ? kNoNeighbour16 : nb[k] - j;
                        if (nb[k] >= 0 && (d < -32767 || d > 32767)) return kTableDoesNotFit;
                        h[k] = (uint32_t)(uint16_t)(int16_t)d;
                    }
                    tab[colour][j] = make_int4((int)(h[0] | h[1] << 16), (int)(h[2] | h[3] << 16),
                                               (int)(h[4] | h[5] << 16), (int)box);
                } else {
                    tab[colour][2 * (size_t)j] = make_int4(nb[0], nb[1], nb[2], nb[3]);
                    tab[colour][2 * (size_t)j + 1] = make_int4(nb[4], nb[5], (int)box, 0);
                }
            }
    for (int colour = 0; colour < 2; ++colour) {
        if (cnt[colour] != c.fill_n[chain * 2 + colour])
            return set_error(NMMC_ERR_ARG, "compact table and filled-site list disagree");
        if (cnt[colour])
            NMMC_CUDA(cudaMemcpy(c.d_ctab + (size_t)(chain * 2 + colour) * NH * per, tab[colour].data(),
                                 tab[colour].size() * sizeof(int4), cudaMemcpyHostToDevice));
    }
    return NMMC_OK;
}

int compact_prepare(Ctx& c) {
    if (!use_compact(c) || c.ctab_built) return NMMC_OK;
    const size_t NH = (size_t)c.m.nhalf, segs = (size_t)c.nchains * 2;
    if (!c.d_cspins) NMMC_CUDA(cudaMalloc(&c.d_cspins, segs * NH * sizeof(float4)));
    for (bool packed : {true, false}) {   // the packed table where every chain's differences fit
        c.ctab_packed = packed;
        cudaFree(c.d_ctab);
        c.d_ctab = nullptr;
        NMMC_CUDA(cudaMalloc(&c.d_ctab, segs * NH * (packed ? 1 : 2) * sizeof(int4)));
        int rc = NMMC_OK;
        for (int ch = 0; ch < c.nchains && rc == NMMC_OK; ++ch) rc = compact_table_chain(c, ch);
        if (rc == kTableDoesNotFit) continue;
        if (rc) return rc;
        c.ctab_built = true;
        return NMMC_OK;
    }
    return set_error(NMMC_ERR_UNSUPPORTED, "compact table could not be built");
}

int launch_global_sweeps(Ctx& c, const int* d_chains, int n, int nsweeps, bool fused) {
    if (use_compact(c)) {
        // filled sites gathered into the compact planes, swept there, and written back
        int rc = compact_prepare(c);
        if (rc) return rc;
        HalfFn fc = c.dim == 3 ? pick_compact<3>(c.m.dmi_kind) : pick_compact<2>(c.m.dmi_kind);
        if ((rc = compact_copy(c, d_chains, n, true))) return rc;
        for (int s = 0; s < nsweeps; ++s)
            for (int colour = 0; colour < 2; ++colour) fc(c, d_chains, n, colour, (unsigned)s);
        if ((rc = cuda_check(cudaGetLastError(), "compact half-sweep launch"))) return rc;
        if ((rc = compact_copy(c, d_chains, n, false))) return rc;
        return launch_advance(c, d_chains, n, nsweeps);
    }
    HalfFn f = pick_half(c);
    HalfFn fm = nullptr;   // the last sweep's colour-1 half-sweep with the observables summed on the way
    if (fused && nsweeps > 0)
        fm = c.dim == 3 ? (c.periodic ? pick_heis_q4_meas<3, true>(c.m.dmi_kind) : pick_heis_q4_meas<3, false>(c.m.dmi_kind))
                        : (c.periodic ? pick_heis_q4_meas<2, true>(c.m.dmi_kind) : pick_heis_q4_meas<2, false>(c.m.dmi_kind));
    // sweeps [w0, w1) as wavefront launches (an even number, so that the result is back in
    // d_spins); the others (the first of an odd count, the fused last one) as half-sweeps
    int w0 = 0, w1 = 0;
    if (wave_ready(c)) {
        w1 = fm ? nsweeps - 1 : nsweeps;
        w0 = w1 & 1;
        if (w1 - w0 < 2) w0 = w1 = 0;
    }
    // the prefetching four-site kernel for plain half-sweeps (NMMC_OPT_HALF_KERNEL 8)
    const bool pf = c.half_kernel == 8 && !c.ising && !c.masked && (c.m.hx % 4) == 0;
    int rc;
    for (int s = 0; s < nsweeps; ++s) {
        if (s >= w0 && s < w1) {
            const bool fwd = ((s - w0) & 1) == 0;
            float* a = (float*)c.d_spins;
            float* b = (float*)c.d_spins_alt;
            if ((rc = launch_wave_sweep(c, fwd ? a : b, fwd ? b : a, d_chains, n, (unsigned)s))) return rc;
            continue;
        }
        for (int colour = 0; colour < 2; ++colour) {
            if (fm && s == nsweeps - 1 && colour == 1) fm(c, d_chains, n, colour, (unsigned)s);
            else if (pf && (rc = launch_pf_half(c, d_chains, n, colour, (unsigned)s))) return rc;
            else if (!pf) f(c, d_chains, n, colour, (unsigned)s);
        }
    }
    rc = cuda_check(cudaGetLastError(), "half-sweep launch");
    if (rc) return rc;
    return launch_advance(c, d_chains, n, nsweeps);
}

// Whether this context's HBM sweeps run as wavefront launches: the option, a lattice the
// kernel covers, the default half-sweep kernel, and the second spin array (allocated here at
// the first call; without the memory for it the context keeps to half-sweeps).
bool wave_ready(Ctx& c) {
    if (!c.wave || c.half_kernel != 0 || c.wave_no_memory || wave_rows(c) == 0) return false;
    if (!c.d_spins_alt && cudaMalloc(&c.d_spins_alt, c.spins_bytes) != cudaSuccess) {
        cudaGetLastError();   // clear the allocation error; half-sweeps from now on
        c.d_spins_alt = nullptr;
        c.wave_no_memory = true;
        return false;
    }
    return true;
}

// Kernel launches of one HBM-path call of nsweeps sweeps (sweeps and counter advance).
long long global_sweep_launches(Ctx& c, int nsweeps, bool fused) {
    if (c.m.general) return (long long)c.m.col_q * nsweeps;
    int waves = 0;
    if (!c.masked && wave_ready(c)) {
        const int w1 = fused ? nsweeps - 1 : nsweeps;
        waves = (w1 - (w1 & 1) >= 2) ? w1 - (w1 & 1) : 0;
    }
    return 2LL * (nsweeps - waves) + waves;
}

// The HBM four-site path can sum E, M, subM and sub4M inside a sample step's last two
// half-sweeps: unmasked Heisenberg lattices of rows with a multiple of 4 sites per colour on
// the default four-site kernel, FP32 observables, and a table whose +-axis records are pairs
// (J(+a) = J(-a), D(-a) = -D(+a)), so that summing the bonds of the colour-1 sites counts
// every bond once.
bool hbm_fused_measure_ok(const Ctx& c) {
    if (c.ising || c.masked || c.m.general || c.measure_fp64 || (c.half_kernel != 0 && c.half_kernel != 8) ||
        (c.m.hx % 4) != 0)
        return false;
    if (c.m.dmi_kind == kDmiGeneral) return false;
    for (int a = 0; a < c.dim; ++a)
        if (c.m.J[2 * a] != c.m.J[2 * a + 1]) return false;
    return true;
}

// ------------------------------------------------------------------------------------------
// Observables (Old/lib/thermodynamics.cpp:71-198)
//
// One block covers `rows` rows of one z-slice of one chain and writes 11 FP64 partials:
// e = sum_i s_i . sum_j (J_ij s_j + D_ij x s_j), M, subM(0), sub4M, and the slice's solid-
// angle sum. Per-site terms are FP32 (or FP64 with NMMC_OPT_MEASURE_FP64) summed per thread
// in the same type; the per-thread totals are combined in FP64 in a fixed order.
// ------------------------------------------------------------------------------------------

template <typename T>
__device__ __forceinline__ T solid_angle_t(T a0, T a1, T a2, T b0, T b1, T b2, T c0, T c1, T c2) {
    // thermodynamics.cpp:200-221 with s1 = a, s2 = b, s3 = c
    T s1s2 = a0 * b0 + a1 * b1 + a2 * b2;
    T s1s3 = a0 * c0 + a1 * c1 + a2 * c2;
    T s2s3 = b0 * c0 + b1 * c1 + b2 * c2;
    T rho = T(2) * (T(1) + s1s2) * (T(1) + s1s3) * (T(1) + s2s3);
    T dotsum = T(1) + s1s2 + s1s3 + s2s3;
    T x0 = a1 * c2 - a2 * c1, x1 = a2 * c0 - a0 * c2, x2 = a0 * c1 - a1 * c0;
    T cross = x0 * b0 + x1 * b1 + x2 * b2;
    return -atan2(cross / rho, dotsum / rho);
}

// FP64 mode: the reference's formula; FP32 mode: its rho -> 0+ limit (above).
__device__ __forceinline__ double solid_angle_sel(double a0, double a1, double a2, double b0, double b1,
                                                  double b2, double c0, double c1, double c2) {
    return solid_angle_t<double>(a0, a1, a2, b0, b1, b2, c0, c1, c2);
}
__device__ __forceinline__ float solid_angle_sel(float a0, float a1, float a2, float b0, float b1, float b2,
                                                 float c0, float c1, float c2) {
    return solid_angle_f(a0, a1, a2, b0, b1, b2, c0, c1, c2);
}

// Block reduction of the per-thread sums in a fixed order, warp sums in the mode's type (FP64
// mode: FP64 throughout; FP32 mode: FP32 warp sums of at most 32 x 16 sites, as k_measure_q4
// and exact for Ising's integer sums), then FP64 across warps on the lanes that own each value
// (the FP64 pipe of this part is narrow: FP64 warp shuffles and adds of every value on every
// warp cost more than the per-site FP32 terms); writes the block's kNP partials to out.
template <typename RT>
__device__ __forceinline__ void block_partials(const RT* acc, double* __restrict__ out) {
    __shared__ RT red[kNP][8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < kNP; ++k) {
        RT v = acc[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[k][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < kNP) {
        double v = 0;
        const int nw = blockDim.x >> 5;
        for (int w = 0; w < nw; ++w) v += (double)red[threadIdx.x][w];
        out[threadIdx.x] = v;
    }
}

// Per-site terms of the observables of the filled site (x, y, z) with spin s and its
// neighbours n (stencil order, 0 where absent) into acc; qv: the neighbours -x, +y and +x, -y
// close the two solid-angle triangles (Old/lib/thermodynamics.cpp:71-198).
template <int DIM, bool ISING, typename RT>
__device__ __forceinline__ void site_terms(const DevModel& m, const int x, const int y, const int z, const RT s0,
                                           const RT s1, const RT s2, const RT* n0, const RT* n1, const RT* n2,
                                           const bool* qv, RT* acc) {
    // energy density (E convention: J s_j + D x s_j)
    RT f0 = RT(0), f1 = RT(0), f2 = RT(0);
#pragma unroll
    for (int k = 0; k < 2 * DIM; ++k) {
        RT J = sizeof(RT) == 8 ? RT(m.Jd[k]) : RT(m.J[k]);
        f0 += J * n0[k];
        if (!ISING) {
            f1 += J * n1[k];
            f2 += J * n2[k];
            if (m.has_dmi) {
                RT d0 = sizeof(RT) == 8 ? RT(m.Ded[k][0]) : RT(m.De[k][0]);
                RT d1 = sizeof(RT) == 8 ? RT(m.Ded[k][1]) : RT(m.De[k][1]);
                RT d2 = sizeof(RT) == 8 ? RT(m.Ded[k][2]) : RT(m.De[k][2]);
                f0 += d1 * n2[k] - d2 * n1[k];
                f1 += d2 * n0[k] - d0 * n2[k];
                f2 += d0 * n1[k] - d1 * n0[k];
            }
        }
    }
    acc[0] += s0 * f0 + s1 * f1 + s2 * f2;
    acc[1] += s0;
    acc[2] += s1;
    acc[3] += s2;
    if (((x + y + z) & 1) == 0) {   // subM(0): (sum of coordinates) % 2 == 0
        acc[4] += s0;
        acc[5] += s1;
        acc[6] += s2;
    }
    {   // sub4M (thermodynamics.cpp:138-163), C truncating remainders
        int kk = (DIM == 3) ? z : 0;
        int possum = x + y;
        int posdiff = -x + y + (m.edge - m.edge % 4);
        bool in4 = (possum % 4 == 0 && posdiff % 4 == 0 && kk % 4 == 0) ||
                   (possum % 4 == 2 && posdiff % 4 == 2 && kk % 4 == 2);
        if (in4) {
            acc[7] += s0;
            acc[8] += s1;
            acc[9] += s2;
        }
    }
    if (!ISING) {   // triangles (i, i-x, i+y) and (i, i+x, i-y)
        if (qv[1] && qv[2])
            acc[10] += solid_angle_sel(s0, s1, s2, n0[1], n1[1], n2[1], n0[2], n1[2], n2[2]);
        if (qv[0] && qv[3])
            acc[10] += solid_angle_sel(s0, s1, s2, n0[0], n1[0], n2[0], n0[3], n1[3], n2[3]);
    }
}

template <int DIM, bool ISING, bool MASKED, typename RT>
__global__ void __launch_bounds__(256)
k_measure(const DevModel m, const void* __restrict__ spins_v, const uint8_t* __restrict__ mask,
          const uint32_t* __restrict__ fill, const int* __restrict__ fill_zoff,
          const int* __restrict__ chains, int rows, int nblk_slice, double* __restrict__ partial) {
    const int ci = blockIdx.y;
    const int chain = chains[ci];
    const int b = blockIdx.x;
    const int z = b / nblk_slice;
    const int y0 = (b - z * nblk_slice) * rows;
    const int y1 = min(y0 + rows, m.ly);
    const int nsite = (y1 - y0) * m.edge;
    const size_t P = (size_t)m.nhalf_pad;
    const int ncomp = ISING ? 1 : 3;
    RT acc[kNP];
#pragma unroll
    for (int k = 0; k < kNP; ++k) acc[k] = RT(0);

    auto filled = [&](int x, int y, int zz) -> bool {
        if (!MASKED) return true;
        int colour = (x + y + zz) & 1;
        return mask[((size_t)chain * 2 + colour) * P + (zz * m.ly + y) * m.hx + (x >> 1)] != 0;
    };
    auto load = [&](int x, int y, int zz, RT& s0, RT& s1, RT& s2) {
        int colour = (x + y + zz) & 1;
        size_t i = (size_t)(zz * m.ly + y) * m.hx + (x >> 1);
        if (ISING) {
            const int8_t* pl = (const int8_t*)spins_v + ((size_t)chain * 2 + colour) * P;
            s0 = RT(pl[i]);
            s1 = s2 = RT(0);
        } else {
            const float* pl = (const float*)spins_v + ((size_t)chain * 2 + colour) * 3 * P;
            s0 = RT(pl[i]);
            s1 = RT(pl[P + i]);
            s2 = RT(pl[2 * P + i]);
        }
    };
    (void)ncomp;

    // terms of the filled site (x, y, z) into acc
    auto site = [&](const int x, const int y, const int z) {
        RT s0, s1, s2;
        load(x, y, z, s0, s1, s2);
        // neighbours in stencil order; wrapped on periodic lattices, absent on open edges
        RT n0[2 * DIM], n1[2 * DIM], n2[2 * DIM];
        bool qv[4];
#pragma unroll
        for (int k = 0; k < 2 * DIM; ++k) {
            int nx = x + (k == 0) - (k == 1), ny = y + (k == 2) - (k == 3), nz = z + (k == 4) - (k == 5);
            bool inside = nx >= 0 && nx < m.edge && ny >= 0 && ny < m.edge && nz >= 0 && nz < m.lz;
            if (m.periodic) {
                nx = (nx + m.edge) % m.edge;
                ny = (ny + m.edge) % m.edge;
                if (DIM == 3) nz = (nz + m.edge) % m.edge;
            }
            bool exists = (m.periodic || inside) && filled(nx, ny, nz);
            if (exists) load(nx, ny, nz, n0[k], n1[k], n2[k]);
            else n0[k] = n1[k] = n2[k] = RT(0);
            if (k < 4) qv[k] = exists && (inside || (m.periodic && m.periodic_q));
        }
        site_terms<DIM, ISING, RT>(m, x, y, z, s0, s1, s2, n0, n1, n2, qv, acc);
    };
    if (MASKED && fill) {
        // part `chunk` of z-slice z's filled sites, both colours, from the chain's lists
        const int chunk = b - z * nblk_slice;
        const int* zo0 = fill_zoff + (size_t)(chain * 2) * (m.lz + 1);
        const int* zo1 = zo0 + (m.lz + 1);
        const int lo0 = zo0[z], cnt0 = zo0[z + 1] - lo0, lo1 = zo1[z], cnt1 = zo1[z + 1] - lo1;
        const int total = cnt0 + cnt1, per = (total + nblk_slice - 1) / nblk_slice;
        const int f1 = min(total, (chunk + 1) * per);
        const uint32_t* l0 = fill + (size_t)(chain * 2) * m.nhalf + lo0;
        const uint32_t* l1 = fill + (size_t)(chain * 2 + 1) * m.nhalf + lo1;
        for (int f = chunk * per + threadIdx.x; f < f1; f += blockDim.x) {
            const int colour = f < cnt0 ? 0 : 1;
            const int i = (int)(colour ? l1[f - cnt0] : l0[f]);
            int x, y, zz;
            decode_site<DIM>(m, i, colour, x, y, zz);
            site(x, y, zz);
        }
    } else {
        for (int t = threadIdx.x; t < nsite; t += blockDim.x) {
            const int yy = t / m.edge;
            const int y = y0 + yy;
            const int x = t - yy * m.edge;
            if (!filled(x, y, z)) continue;
            site(x, y, z);
        }
    }
    block_partials<RT>(acc, partial + ((size_t)ci * gridDim.x + b) * kNP);
}

// Heisenberg observables over quads of same-colour sites (unmasked lattices, rows holding a
// multiple of 4 sites per colour): the neighbour loads of the sweep kernel feed the energy
// density, M, subM(0), sub4M and both solid-angle triangles of every site. FP32 per-site
// terms; the partial-sum layout is that of k_measure. The energy density takes the DMI
// structure of the model (DK, as the sweep): for +-axis pairs with De(-a) = -De(+a),
// J (n+ + n-) + De(+a) x (n+ - n-), which is the per-direction sum regrouped.
// SPT consecutive same-colour sites per thread item: 2 (float2 rows, 64 registers, 4 CTAs/SM;
// the default, measured fastest on the benchmark lattice) or 4 (float4 rows, 128 registers,
// 2 CTAs/SM); the same per-site terms, summed per thread in another order.
// QONLY: the topological charge alone (the other ten partials written as 0): the pass that
// follows the fused half-sweep of nmmc_sweep_measure, which summed E, M, subM and sub4M.
template <int DIM, bool PERIODIC, int DK, int SPT, bool QONLY = false>
__global__ void __launch_bounds__(256, SPT == 4 ? (QONLY ? 3 : 2) : 4)
k_measure_q4(const DevModel m, const float* __restrict__ spins, const int* __restrict__ chains, int rows,
             int nblk_slice, double* __restrict__ partial) {
    const int ci = blockIdx.y;
    const int chain = chains[ci];
    const int b = blockIdx.x;
    const int z = b / nblk_slice;
    const int y0 = (b - z * nblk_slice) * rows;
    const int y1 = min(y0 + rows, m.ly);
    using VT = typename SiteVec<SPT>::T;
    const int qpr = m.hx / SPT;
    const int qshift = (m.qpr_shift >= 0) ? m.qpr_shift + (SPT == 2 ? 1 : 0) : -1;   // log2(hx / SPT)
    const int nitem = 2 * (y1 - y0) * qpr;
    const size_t P = (size_t)m.nhalf_pad;
    const bool pq = PERIODIC && m.periodic_q;
    const int e4 = m.edge - m.edge % 4;
    float acc[kNP];
#pragma unroll
    for (int k = 0; k < kNP; ++k) acc[k] = 0.0f;

    for (int it = threadIdx.x; it < nitem; it += blockDim.x) {
        const int colour = it & 1;
        const int rq = it >> 1;
        const int yy = (qshift >= 0) ? (rq >> qshift) : (rq / qpr);
        const int h0 = (rq - yy * qpr) * SPT;
        const int y = y0 + yy;
        const int row = z * m.ly + y;
        const int xp = (y + z + colour) & 1;
        const float* own = spins + ((size_t)chain * 2 + colour) * 3 * P;
        const float* oth = spins + ((size_t)chain * 2 + (colour ^ 1)) * 3 * P;
        const int rb = row * m.hx + h0;
        VT s[3], same[3], yp[3], ym[3], zp[3], zm[3];
        const VT vz = {};
        float ex[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            s[c] = __ldg(reinterpret_cast<const VT*>(own + c * P + rb));
            same[c] = __ldg(reinterpret_cast<const VT*>(oth + c * P + rb));
        }
        int hx_out = xp ? h0 + SPT : h0 - 1;
        bool ex_ok = true;
        if (PERIODIC) hx_out = (hx_out < 0) ? m.hx - 1 : (hx_out >= m.hx ? 0 : hx_out);
        else ex_ok = hx_out >= 0 && hx_out < m.hx;
#pragma unroll
        for (int c = 0; c < 3; ++c) ex[c] = ex_ok ? __ldg(oth + c * P + row * m.hx + hx_out) : 0.0f;
        int yu = y + 1, yd = y - 1;
        bool okU = true, okD = true;
        if (PERIODIC) {
            yu = (yu == m.edge) ? 0 : yu;
            yd = (yd < 0) ? m.edge - 1 : yd;
        } else {
            okU = yu < m.edge;
            okD = yd >= 0;
        }
        {
            const int ru = (z * m.ly + yu) * m.hx + h0, rd = (z * m.ly + yd) * m.hx + h0;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                yp[c] = okU ? __ldg(reinterpret_cast<const VT*>(oth + c * P + ru)) : vz;
                ym[c] = okD ? __ldg(reinterpret_cast<const VT*>(oth + c * P + rd)) : vz;
            }
        }
        if (QONLY) {
#pragma unroll
            for (int c = 0; c < 3; ++c) zp[c] = zm[c] = vz;
        } else if (DIM == 3) {
            int zu = z + 1, zd = z - 1;
            bool oU = true, oD = true;
            if (PERIODIC) {
                zu = (zu == m.edge) ? 0 : zu;
                zd = (zd < 0) ? m.edge - 1 : zd;
            } else {
                oU = zu < m.lz;
                oD = zd >= 0;
            }
            const int ru = (zu * m.ly + y) * m.hx + h0, rd = (zd * m.ly + y) * m.hx + h0;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                zp[c] = oU ? __ldg(reinterpret_cast<const VT*>(oth + c * P + ru)) : vz;
                zm[c] = oD ? __ldg(reinterpret_cast<const VT*>(oth + c * P + rd)) : vz;
            }
        }
        // triangles use the unwrapped in-plane adjacency unless periodic_q
        const bool qyu = okU && (y + 1 < m.edge || pq), qyd = okD && (y >= 1 || pq);
#pragma unroll
        for (int k = 0; k < SPT; ++k) {
            const int x = 2 * (h0 + k) + xp;
            float n0[6], n1[6], n2[6];
            float* nn[3] = {n0, n1, n2};
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                float sm = vel(same[c], k);
                float sh = xp ? (k < SPT - 1 ? vel(same[c], k + 1) : ex[c]) : (k > 0 ? vel(same[c], k - 1) : ex[c]);
                float plusx = xp ? sh : sm, minusx = xp ? sm : sh;
                if (!PERIODIC) {
                    if (x + 1 >= m.edge) plusx = 0.0f;
                    if (x == 0) minusx = 0.0f;
                }
                nn[c][0] = plusx;
                nn[c][1] = minusx;
                nn[c][2] = vel(yp[c], k);
                nn[c][3] = vel(ym[c], k);
                if (DIM == 3) {
                    nn[c][4] = vel(zp[c], k);
                    nn[c][5] = vel(zm[c], k);
                }
            }
            const float s0 = vel(s[0], k), s1 = vel(s[1], k), s2 = vel(s[2], k);
            float f0 = 0.f, f1 = 0.f, f2 = 0.f;
            if (QONLY) {
            } else if (DK <= kDmiGeneral) {
#pragma unroll
                for (int d = 0; d < 2 * DIM; ++d) {
                    const float J = m.J[d];
                    f0 = fmaf(J, n0[d], f0);
                    f1 = fmaf(J, n1[d], f1);
                    f2 = fmaf(J, n2[d], f2);
                    if (DK == kDmiGeneral) {   // D x s_j
                        f0 = fmaf(m.De[d][1], n2[d], fmaf(-m.De[d][2], n1[d], f0));
                        f1 = fmaf(m.De[d][2], n0[d], fmaf(-m.De[d][0], n2[d], f1));
                        f2 = fmaf(m.De[d][0], n1[d], fmaf(-m.De[d][1], n0[d], f2));
                    }
                }
            } else {
#pragma unroll
                for (int a = 0; a < DIM; ++a) {
                    const int kp = 2 * a, km = 2 * a + 1;
                    const float J = m.J[kp];
                    f0 = fmaf(J, n0[kp] + n0[km], f0);
                    f1 = fmaf(J, n1[kp] + n1[km], f1);
                    f2 = fmaf(J, n2[kp] + n2[km], f2);
                    const float d0 = n0[kp] - n0[km], d1 = n1[kp] - n1[km], d2 = n2[kp] - n2[km];
                    if (DK == kDmiPairs) {   // De(+a) x d
                        f0 = fmaf(m.De[kp][1], d2, fmaf(-m.De[kp][2], d1, f0));
                        f1 = fmaf(m.De[kp][2], d0, fmaf(-m.De[kp][0], d2, f1));
                        f2 = fmaf(m.De[kp][0], d1, fmaf(-m.De[kp][1], d0, f2));
                    } else {                 // De(+a) = D e_a: D (e_a x d)
                        const float D = m.De[kp][a];
                        if (a == 0) {
                            f1 = fmaf(-D, d2, f1);
                            f2 = fmaf(D, d1, f2);
                        } else if (a == 1) {
                            f0 = fmaf(D, d2, f0);
                            f2 = fmaf(-D, d0, f2);
                        } else {
                            f0 = fmaf(-D, d1, f0);
                            f1 = fmaf(D, d0, f1);
                        }
                    }
                }
            }
            if (!QONLY) {
                acc[0] = fmaf(s0, f0, fmaf(s1, f1, fmaf(s2, f2, acc[0])));
                acc[1] += s0;
                acc[2] += s1;
                acc[3] += s2;
                if (colour == 0) {
                    acc[4] += s0;
                    acc[5] += s1;
                    acc[6] += s2;
                }
                const int possum = x + y, posdiff = -x + y + e4, kk = (DIM == 3) ? z : 0;
                if ((possum % 4 == 0 && posdiff % 4 == 0 && kk % 4 == 0) ||
                    (possum % 4 == 2 && posdiff % 4 == 2 && kk % 4 == 2)) {
                    acc[7] += s0;
                    acc[8] += s1;
                    acc[9] += s2;
                }
            }
            const bool qxm = (x >= 1 || pq), qxp = (x + 1 < m.edge || pq);
            if (qxm && qyu)
                acc[10] += solid_angle_f(s0, s1, s2, n0[1], n1[1], n2[1], n0[2], n1[2], n2[2]);
            if (qxp && qyd)
                acc[10] += solid_angle_f(s0, s1, s2, n0[0], n1[0], n2[0], n0[3], n1[3], n2[3]);
        }
    }
    // warp sums in FP32 (at most 32 x 16 per-site terms), then FP64 across warps: the FP64
    // pipe of this part is narrow, so the warp sums are kept in FP32 and each is converted
    // (exactly) and added by the lane that owns its value: 2 x 8 FP64 warp instructions per
    // block, where converting on each warp's lane 0 took 11 per warp
    if (QONLY) {   // only the solid-angle sum is not zero
        float qv[1] = {acc[10]};
        double* out = partial + ((size_t)ci * gridDim.x + b) * kNP;
        if (threadIdx.x < kNP - 1) out[threadIdx.x] = 0.0;
        meas_block_rows<1>(qv, out + 10);
        return;
    }
    __shared__ float red[kNP][8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < kNP; ++k) {
        float v = acc[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[k][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < kNP) {
        double v = 0;
        const int nw = blockDim.x >> 5;
        for (int w = 0; w < nw; ++w) v += (double)red[threadIdx.x][w];
        partial[((size_t)ci * gridDim.x + b) * kNP + threadIdx.x] = v;
    }
}

// One row of a charge strip: the four sites x = 4j .. 4j+3 of row y of slice z (u[site][comp]);
// the even-x sites are colour (y + z) & 1, the odd ones the other colour: one 8-byte load per
// colour plane and component.
__device__ __forceinline__ void charge_row(const DevModel& m, const float* c0, const float* c1, size_t P, int z,
                                           int y, int h0, float (&u)[4][3]) {
    const bool swap = (y + z) & 1;
    const float* pe = swap ? c1 : c0;
    const float* po = swap ? c0 : c1;
    const size_t rb = (size_t)(z * m.ly + y) * m.hx + h0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float2 ve = __ldg(reinterpret_cast<const float2*>(pe + k * P + rb));
        const float2 vo = __ldg(reinterpret_cast<const float2*>(po + k * P + rb));
        u[0][k] = ve.x;
        u[1][k] = vo.x;
        u[2][k] = ve.y;
        u[3][k] = vo.y;
    }
}

// The strip's x-neighbours in row y: x = 4j - 1 (odd, compact index hl) and x = 4j + 4 (even,
// hr), already wrapped.
__device__ __forceinline__ void charge_edges(const DevModel& m, const float* c0, const float* c1, size_t P, int z,
                                             int y, int hl, int hr, float (&el)[3], float (&er)[3]) {
    const bool swap = (y + z) & 1;
    const float* pe = swap ? c1 : c0;
    const float* po = swap ? c0 : c1;
    const size_t rb = (size_t)(z * m.ly + y) * m.hx;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        el[k] = __ldg(po + k * P + rb + hl);
        er[k] = __ldg(pe + k * P + rb + hr);
    }
}

// The topological charge alone by sliding rows: the pass that follows the fused half-sweep of
// nmmc_sweep_measure on the HBM four-site path (unmasked lattices, edge a multiple of 4 up to
// 1024). A thread owns a strip of four consecutive sites of a row, x = 4j .. 4j+3, and walks
// R rows of one slice keeping rows y-1, y and y+1 in registers, so each spin is loaded about
// once per pass (plus the strip's two x-neighbours and the segment's two boundary rows), where
// the charge-only items of k_measure_q4 load it as an own site, a same-row neighbour and both
// y-neighbours. The triangles are those of calc_TC (Old/lib/thermodynamics.cpp:165-198):
// T1(i) = (s_i, s_{i-x}, s_{i+y}) and T2(i) = (s_i, s_{i+x}, s_{i-y}), with the same inclusion
// rules as k_measure_q4 (unwrapped unless periodic_q). The dot product of a bond is computed
// once for the two triangles that share it (the same FP32 value either way), so every angle
// equals k_measure_q4's bit for bit; only the FP32 summation order differs. Row y's T2
// triangles, which do not need row y+1, are computed while row y+1's loads are in flight.
// Block b of chain item ci covers rows [(b % nblk_slice) * nseg * R, + nseg * R) of slice
// b / nblk_slice: threadIdx = segment * nstrip + strip. Partials in k_measure's layout (the
// ten non-charge entries 0).
template <bool PERIODIC>
__global__ void __launch_bounds__(256, 3)
k_charge_rows(const DevModel m, const float* __restrict__ spins, const int* __restrict__ chains, int nstrip,
              int nseg, int R, int nblk_slice, double* __restrict__ partial) {
    const int ci = blockIdx.y;
    const int chain = chains[ci];
    const int b = blockIdx.x;
    const int z = b / nblk_slice;
    const int j = threadIdx.x % nstrip, g = threadIdx.x / nstrip;
    const int ya = ((b - z * nblk_slice) * nseg + g) * R;
    const int yb = min(ya + R, m.ly);
    float acc = 0.0f;
    if (g < nseg && ya < m.ly) {
        const size_t P = (size_t)m.nhalf_pad;
        const float* c0 = spins + (size_t)chain * 6 * P;
        const float* c1 = c0 + 3 * P;
        const bool pq = PERIODIC && m.periodic_q;
        const int h0 = 2 * j;
        const int hl = (h0 == 0) ? m.hx - 1 : h0 - 1;
        const int hr = (h0 + 2 == m.hx) ? 0 : h0 + 2;
        const bool qx_first = j > 0 || pq;                // T1 of x = 4j has its x - 1
        const bool qx_last = 4 * j + 4 < m.edge || pq;    // T2 of x = 4j + 3 has its x + 1
        float dn[4][3], cu[4][3], up[4][3];
        float cl[3], cr[3];
        float dyp[4];
        {
            int yd = ya - 1;
            bool okD = true;
            if (PERIODIC) yd = (yd < 0) ? m.ly - 1 : yd;
            else okD = yd >= 0;
            if (okD) {
                charge_row(m, c0, c1, P, z, yd, h0, dn);
            } else {
#pragma unroll
                for (int u = 0; u < 4; ++u) dn[u][0] = dn[u][1] = dn[u][2] = 0.0f;
            }
        }
        charge_row(m, c0, c1, P, z, ya, h0, cu);
#pragma unroll
        for (int u = 0; u < 4; ++u) dyp[u] = dot3f(dn[u][0], dn[u][1], dn[u][2], cu[u][0], cu[u][1], cu[u][2]);
        // unrolled by the rotation period of the three rows, so that the rotation is a renaming
        // of registers rather than 28 moves per row (318 against 347 us per 40-chain launch)
#pragma unroll 3
        for (int y = ya; y < yb; ++y) {
            int yu = y + 1;
            bool okU = true;
            if (PERIODIC) yu = (yu == m.ly) ? 0 : yu;
            else okU = yu < m.ly;
            charge_edges(m, c0, c1, P, z, y, hl, hr, cl, cr);
            if (okU) {
                charge_row(m, c0, c1, P, z, yu, h0, up);
            } else {
#pragma unroll
                for (int u = 0; u < 4; ++u) up[u][0] = up[u][1] = up[u][2] = 0.0f;
            }
            const bool qyu = y + 1 < m.ly || pq, qyd = y >= 1 || pq;
            // x-bond products of row y: dx[k] = s(4j - 1 + k) . s(4j + k)
            float dx[5];
            dx[0] = dot3f(cl[0], cl[1], cl[2], cu[0][0], cu[0][1], cu[0][2]);
#pragma unroll
            for (int k = 1; k < 4; ++k)
                dx[k] = dot3f(cu[k - 1][0], cu[k - 1][1], cu[k - 1][2], cu[k][0], cu[k][1], cu[k][2]);
            dx[4] = dot3f(cu[3][0], cu[3][1], cu[3][2], cr[0], cr[1], cr[2]);
            if (qyd) {   // T2: (s, s + x, s - y)
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    if (u == 3 && !qx_last) continue;
                    const float r0 = u < 3 ? cu[u + 1][0] : cr[0];
                    const float r1 = u < 3 ? cu[u + 1][1] : cr[1];
                    const float r2 = u < 3 ? cu[u + 1][2] : cr[2];
                    acc += solid_angle_dots(cu[u][0], cu[u][1], cu[u][2], r0, r1, r2, dn[u][0], dn[u][1], dn[u][2],
                                            dx[u + 1], dyp[u], dot3f(r0, r1, r2, dn[u][0], dn[u][1], dn[u][2]));
                }
            }
            float dyc[4];
#pragma unroll
            for (int u = 0; u < 4; ++u)
                dyc[u] = dot3f(cu[u][0], cu[u][1], cu[u][2], up[u][0], up[u][1], up[u][2]);
            if (qyu) {   // T1: (s, s - x, s + y)
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    if (u == 0 && !qx_first) continue;
                    const float l0 = u > 0 ? cu[u - 1][0] : cl[0];
                    const float l1 = u > 0 ? cu[u - 1][1] : cl[1];
                    const float l2 = u > 0 ? cu[u - 1][2] : cl[2];
                    acc += solid_angle_dots(cu[u][0], cu[u][1], cu[u][2], l0, l1, l2, up[u][0], up[u][1], up[u][2],
                                            dx[u], dyc[u], dot3f(l0, l1, l2, up[u][0], up[u][1], up[u][2]));
                }
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                dyp[u] = dyc[u];
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    dn[u][k] = cu[u][k];
                    cu[u][k] = up[u][k];
                }
            }
        }
    }
    const float qv[1] = {acc};
    double* out = partial + ((size_t)ci * gridDim.x + b) * kNP;
    if (threadIdx.x < kNP - 1) out[threadIdx.x] = 0.0;
    meas_block_rows<1>(qv, out + 10);
}

__global__ void k_measure_finalize(const int* __restrict__ chains, int nblk, int nblk_slice,
                                   int nslices, int ising, const double* __restrict__ partial,
                                   const double* __restrict__ Hd, double* __restrict__ obs,
                                   double* __restrict__ q, double* __restrict__ accum,
                                   int accumulate) {
    const int ci = blockIdx.x;
    const int chain = chains[ci];
    const int lane = threadIdx.x;
    const double* pp = partial + (size_t)ci * nblk * kNP;
    double mine = 0;   // lane k: total k
#pragma unroll
    for (int k = 0; k < kNP - 1; ++k) {
        double v = 0;
        for (int b = lane; b < nblk; b += 32) v += pp[(size_t)b * kNP + k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        const double t = __shfl_sync(0xffffffffu, v, 0);
        if (lane == k) mine = t;
    }
    // per-slice topological charge
    double qsum = 0;
    for (int zs = lane; zs < nslices; zs += 32) {
        double v = 0;
        for (int b = 0; b < nblk_slice; ++b) v += pp[((size_t)zs * nblk_slice + b) * kNP + 10];
        v = ising ? 0.0 : v / (2 * M_PI);
        if (q) q[(size_t)ci * nslices + zs] = v;
        qsum += v;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) qsum += __shfl_down_sync(0xffffffffu, qsum, o);
    qsum = __shfl_sync(0xffffffffu, qsum, 0);
    finalize_chain_warp(mine, lane, Hd + 3 * (size_t)chain, qsum, obs + (size_t)ci * NMMC_OBS_N,
                        accum + (size_t)chain * NMMC_ACC_N, accumulate);
}

// Per-chain finish of nmmc_sweep_measure's fused form on the HBM four-site path: the totals
// come from the block rows of the fused colour-1 half-sweep (2 e, M of colour 1, M of colour
// 0 = submag(0), sub4M), the per-slice charge from the charge pass's partials (the layout of
// k_measure_finalize). One block of 256 threads per chain: each thread sums a fixed stride of
// rows in FP64, then a fixed-order tree across the block, then one warp finishes the chain.
__global__ void __launch_bounds__(256)
k_measure_finalize_fused(const int* __restrict__ chains, const double* __restrict__ qpart, int nblk_q,
                         int nblk_slice, int nslices, const double* __restrict__ rows, int nrows,
                         const double* __restrict__ Hd,
                         double* __restrict__ obs, double* __restrict__ q, double* __restrict__ accum,
                         int accumulate) {
    const int ci = blockIdx.x;
    const int chain = chains[ci];
    const double* B = rows + (size_t)ci * nrows * 10;
    // t: 0 e, 1-3 M, 4-6 subM, 7-9 sub4M
    double t[10];
#pragma unroll
    for (int k = 0; k < 10; ++k) t[k] = 0.0;
    for (int r = threadIdx.x; r < nrows; r += blockDim.x) {
        const double* bb = B + (size_t)r * 10;   // 2 e, M of colour 1, M of colour 0, sub4M
        t[0] += bb[0];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            t[1 + c] += bb[4 + c] + bb[1 + c];
            t[4 + c] += bb[4 + c];
            t[7 + c] += bb[7 + c];
        }
    }
    __shared__ double red[10][256];
#pragma unroll
    for (int k = 0; k < 10; ++k) red[k][threadIdx.x] = t[k];
    __syncthreads();
    for (int w = blockDim.x / 2; w >= 32; w >>= 1) {
        if ((int)threadIdx.x < w)
#pragma unroll
            for (int k = 0; k < 10; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x >= 32) return;
    const int lane = threadIdx.x;
    double mine = 0;   // lane k: total k
#pragma unroll
    for (int k = 0; k < 10; ++k) {
        double v = red[k][lane];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        const double tv = __shfl_sync(0xffffffffu, v, 0);
        if (lane == k) mine = tv;
    }
    const double* pp = qpart + (size_t)ci * nblk_q * kNP;
    double qsum = 0;
    for (int zs = lane; zs < nslices; zs += 32) {
        double v = 0;
        for (int b = 0; b < nblk_slice; ++b) v += pp[((size_t)zs * nblk_slice + b) * kNP + 10];
        v = v / (2 * M_PI);
        if (q) q[(size_t)ci * nslices + zs] = v;
        qsum += v;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) qsum += __shfl_down_sync(0xffffffffu, qsum, o);
    qsum = __shfl_sync(0xffffffffu, qsum, 0);
    finalize_chain_warp(mine, lane, Hd + 3 * (size_t)chain, qsum, obs + (size_t)ci * NMMC_OBS_N,
                        accum + (size_t)chain * NMMC_ACC_N, accumulate);
}

// Masked Heisenberg lattices whose compact form is built (FP32 observables): the blocks of
// k_measure's list split (part `chunk` of z-slice z's filled sites, both colours, in list
// order) over the compact planes, gathered from the box layout just before, with neighbours
// from the compact table. The same per-site terms of the same values in the same order as
// k_measure, so the same sums; the dense planes spare the box layout's part-empty sectors.
template <int DIM, bool PACKED>
__global__ void __launch_bounds__(256)
k_measure_compact(const DevModel m, const float4* __restrict__ cs, const int4* __restrict__ tab,
                  const int* __restrict__ fill_zoff, const int* __restrict__ chains, int nblk_slice,
                  double* __restrict__ partial) {
    const int ci = blockIdx.y;
    const int chain = chains[ci];
    const int b = blockIdx.x;
    const int z = b / nblk_slice;
    const size_t NH = (size_t)m.nhalf;
    float acc[kNP];
#pragma unroll
    for (int k = 0; k < kNP; ++k) acc[k] = 0.0f;
    const int chunk = b - z * nblk_slice;
    const int* zo0 = fill_zoff + (size_t)(chain * 2) * (m.lz + 1);
    const int* zo1 = zo0 + (m.lz + 1);
    const int lo0 = zo0[z], cnt0 = zo0[z + 1] - lo0, lo1 = zo1[z], cnt1 = zo1[z + 1] - lo1;
    const int total = cnt0 + cnt1, per = (total + nblk_slice - 1) / nblk_slice;
    const int f1 = min(total, (chunk + 1) * per);
    for (int f = chunk * per + threadIdx.x; f < f1; f += blockDim.x) {
        const int colour = f < cnt0 ? 0 : 1;
        const int j = colour ? lo1 + (f - cnt0) : lo0 + f;
        const int seg = chain * 2 + colour;
        int nbi[6];
        uint32_t box;
        compact_entry<PACKED>(tab, seg, NH, j, nbi, box);
        const float4* own = cs + (size_t)seg * NH;
        const float4* oth = cs + (size_t)(chain * 2 + (colour ^ 1)) * NH;
        const int x = (int)(box % (uint32_t)m.edge), y = (int)((box / (uint32_t)m.edge) % (uint32_t)m.edge);
        const int zz = (DIM == 3) ? (int)(box / ((uint32_t)m.edge * (uint32_t)m.edge)) : 0;
        const float4 sv = own[j];
        const float s0 = sv.x, s1 = sv.y, s2 = sv.z;
        float n0[2 * DIM], n1[2 * DIM], n2[2 * DIM];
        bool qv[4];
#pragma unroll
        for (int k = 0; k < 2 * DIM; ++k) {
            const int q = nbi[k];
            const bool exists = q >= 0;
            const float4 v = exists ? __ldg(oth + q) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            n0[k] = v.x;
            n1[k] = v.y;
            n2[k] = v.z;
            if (k < 4) {
                const int nx = x + (k == 0) - (k == 1), ny = y + (k == 2) - (k == 3);
                const bool inside = nx >= 0 && nx < m.edge && ny >= 0 && ny < m.edge;
                qv[k] = exists && (inside || (m.periodic && m.periodic_q));
            }
        }
        site_terms<DIM, false, float>(m, x, y, zz, s0, s1, s2, n0, n1, n2, qv, acc);
    }
    block_partials<float>(acc, partial + ((size_t)ci * gridDim.x + b) * kNP);
}

template <int DIM, bool PER, int SPT>
static void measure_q4_spt(Ctx& c, dim3 grid, const float* sp, const int* d_chains, int rows, int nblk_slice,
                           double* partial) {
    switch (c.m.dmi_kind) {
        case kDmiNone:
            k_measure_q4<DIM, PER, kDmiNone, SPT><<<grid, 256, 0, c.stream>>>(c.m, sp, d_chains, rows, nblk_slice, partial);
            break;
        case kDmiGeneral:
            k_measure_q4<DIM, PER, kDmiGeneral, SPT><<<grid, 256, 0, c.stream>>>(c.m, sp, d_chains, rows, nblk_slice,
                                                                               partial);
            break;
        case kDmiPairs:
            k_measure_q4<DIM, PER, kDmiPairs, SPT><<<grid, 256, 0, c.stream>>>(c.m, sp, d_chains, rows, nblk_slice, partial);
            break;
        default:
            k_measure_q4<DIM, PER, kDmiAxial, SPT><<<grid, 256, 0, c.stream>>>(c.m, sp, d_chains, rows, nblk_slice, partial);
            break;
    }
}

template <int DIM, bool PER>
static void measure_q4_dk(Ctx& c, dim3 grid, const float* sp, const int* d_chains, int rows, int nblk_slice,
                          double* partial) {
    if (c.measure_sites == 2) measure_q4_spt<DIM, PER, 2>(c, grid, sp, d_chains, rows, nblk_slice, partial);
    else measure_q4_spt<DIM, PER, 4>(c, grid, sp, d_chains, rows, nblk_slice, partial);
}

static void measure_q4_launch(Ctx& c, dim3 grid, const float* sp, const int* d_chains, int rows, int nblk_slice,
                              double* partial) {
    if (c.dim == 3) {
        if (c.periodic) measure_q4_dk<3, true>(c, grid, sp, d_chains, rows, nblk_slice, partial);
        else measure_q4_dk<3, false>(c, grid, sp, d_chains, rows, nblk_slice, partial);
    } else {
        if (c.periodic) measure_q4_dk<2, true>(c, grid, sp, d_chains, rows, nblk_slice, partial);
        else measure_q4_dk<2, false>(c, grid, sp, d_chains, rows, nblk_slice, partial);
    }
}

// Masked lattices are measured over their lists of filled sites (blocks = parts of z-slices),
// except with a general interaction table, whose energy kernel adds into the partial sums of
// the row-split blocks.
static bool measure_by_list(const Ctx& c) { return c.masked && !c.m.general && c.d_fill; }

// FP32 observables of masked Heisenberg lattices whose compact form is built: the list split
// over the compact planes (gathered from the box layout first).
static bool measure_by_compact(const Ctx& c) {
    return measure_by_list(c) && use_compact(c) && c.ctab_built && !c.measure_fp64;
}

static int measure_compact_launch(Ctx& c, const int* d_chains, int n, int nblk, int nblk_slice, double* partial) {
    int rc = compact_copy(c, d_chains, n, true);
    if (rc) return rc;
    dim3 grid(nblk, n);
#define NMMC_MC(D, PK) k_measure_compact<D, PK><<<grid, 256, 0, c.stream>>>(c.m, c.d_cspins, c.d_ctab, \
                                                                             c.d_fill_zoff, d_chains, nblk_slice, partial)
    if (c.dim == 3) { if (c.ctab_packed) NMMC_MC(3, true); else NMMC_MC(3, false); }
    else { if (c.ctab_packed) NMMC_MC(2, true); else NMMC_MC(2, false); }
#undef NMMC_MC
    return NMMC_OK;
}

template <int DIM, bool ISING, bool MASKED>
static void measure_launch(Ctx& c, const int* d_chains, int n, int rows, int nblk_slice, bool fp64, double* partial) {
    dim3 grid(nblk_slice * c.m.lz, n);
    const uint32_t* fill = measure_by_list(c) ? c.d_fill : nullptr;
    if (fp64)
        k_measure<DIM, ISING, MASKED, double><<<grid, 256, 0, c.stream>>>(
            c.m, c.d_spins, c.d_mask, fill, c.d_fill_zoff, d_chains, rows, nblk_slice, partial);
    else
        k_measure<DIM, ISING, MASKED, float><<<grid, 256, 0, c.stream>>>(
            c.m, c.d_spins, c.d_mask, fill, c.d_fill_zoff, d_chains, rows, nblk_slice, partial);
}

struct MeasureShape {
    int rows, nblk_slice, nblk;
};

static MeasureShape measure_shape(const Ctx& c) {
    // about 4096 sites per block: rows of one z-slice, or a part of one z-slice's filled sites
    MeasureShape s;
    if (measure_by_list(c)) {
        s.rows = c.m.ly;
        s.nblk_slice = std::max(1, (c.fill_slice_max + 4095) / 4096);
    } else {
        s.rows = 4096 / c.edge;
        if (s.rows < 1) s.rows = 1;
        if (s.rows > c.m.ly) s.rows = c.m.ly;
        s.nblk_slice = (c.m.ly + s.rows - 1) / s.rows;
    }
    s.nblk = s.nblk_slice * c.m.lz;
    return s;
}

size_t measure_partials_per_chain(const Ctx& c) { return (size_t)measure_shape(c).nblk * kNP; }

// Sizes the partial-sum scratch for n chains (allocation is not allowed during capture).
int measure_prepare(Ctx& c, int n) {
    size_t need = (size_t)n * measure_partials_per_chain(c);
    if (need > c.partial_cap) {
        if (c.d_partial) cudaFree(c.d_partial);
        c.d_partial = nullptr;
        c.partial_cap = 0;
        NMMC_CUDA(cudaMalloc(&c.d_partial, need * sizeof(double)));
        c.partial_cap = need;
    }
    // block rows of the fused half-sweep (lattices that could take that form)
    if (!c.ising && !c.masked && !c.m.general && (c.m.hx % 4) == 0) {
        const size_t rows = (size_t)n * q4_meas_blocks(c) * 10;
        if (rows > c.mrows_cap) {
            if (c.d_mrows) cudaFree(c.d_mrows);
            c.d_mrows = nullptr;
            c.mrows_cap = 0;
            NMMC_CUDA(cudaMalloc(&c.d_mrows, rows * sizeof(double)));
            c.mrows_cap = rows;
        }
    }
    return NMMC_OK;
}

// The measurement kernels of the listed chains with their per-block partial sums in
// `partial` (n * measure_partials_per_chain(c) doubles, every slot written before it is
// read), then the per-chain finish into obs / q (and the accumulators when asked).
static int measure_with(Ctx& c, const int* d_chains, int n, double* partial, double* obs, double* q,
                        int accumulate) {
    const MeasureShape ms = measure_shape(c);
    const int rows = ms.rows, nblk_slice = ms.nblk_slice, nblk = ms.nblk;
    const bool fp64 = c.measure_fp64 != 0;
    if (measure_by_compact(c)) {
        int rc = measure_compact_launch(c, d_chains, n, nblk, nblk_slice, partial);
        if (rc) return rc;
    } else if (!c.ising && !c.masked && !fp64 && (c.m.hx % 4) == 0 && c.half_kernel != 1 && !c.m.general) {
        dim3 grid(nblk, n);
        const float* sp = (const float*)c.d_spins;
        measure_q4_launch(c, grid, sp, d_chains, rows, nblk_slice, partial);
    } else if (c.ising) {
        if (c.dim == 3) c.masked ? measure_launch<3, true, true>(c, d_chains, n, rows, nblk_slice, fp64, partial)
                                 : measure_launch<3, true, false>(c, d_chains, n, rows, nblk_slice, fp64, partial);
        else c.masked ? measure_launch<2, true, true>(c, d_chains, n, rows, nblk_slice, fp64, partial)
                      : measure_launch<2, true, false>(c, d_chains, n, rows, nblk_slice, fp64, partial);
    } else {
        if (c.dim == 3) c.masked ? measure_launch<3, false, true>(c, d_chains, n, rows, nblk_slice, fp64, partial)
                                 : measure_launch<3, false, false>(c, d_chains, n, rows, nblk_slice, fp64, partial);
        else c.masked ? measure_launch<2, false, true>(c, d_chains, n, rows, nblk_slice, fp64, partial)
                      : measure_launch<2, false, false>(c, d_chains, n, rows, nblk_slice, fp64, partial);
    }
    if (c.m.general) {   // the general table's energy term, added to the same partial sums
        int rc = launch_energy_general(c, d_chains, n, rows, nblk_slice, nblk, partial);
        if (rc) return rc;
    }
    k_measure_finalize<<<n, 32, 0, c.stream>>>(d_chains, nblk, nblk_slice, c.m.lz, c.ising ? 1 : 0, partial,
                                               c.d_Hd, obs, q, c.d_acc, accumulate);
    return cuda_check(cudaGetLastError(), "measure launch");
}

int launch_measure(Ctx& c, const int* d_chains, int n, int accumulate) {
    if ((size_t)n * measure_partials_per_chain(c) > c.partial_cap) {
        int rc = measure_prepare(c, n);
        if (rc) return rc;
    }
    return measure_with(c, d_chains, n, c.d_partial, c.d_obs, c.d_q, accumulate);
}

int hbm_tuning_step(Ctx& c, int nsweeps, bool measure) {
    int rc;
    if (measure && hbm_fused_measure_ok(c)) {
        if ((rc = measure_prepare(c, c.nchains))) return rc;
        if ((rc = launch_global_sweeps(c, c.d_all, c.nchains, nsweeps, true))) return rc;
        return launch_measure_fused_tail(c, c.d_all, c.nchains, 0);
    }
    if ((rc = launch_global_sweeps(c, c.d_all, c.nchains, nsweeps, false))) return rc;
    return measure ? launch_measure(c, c.d_all, c.nchains, 0) : NMMC_OK;
}

// After the fused last sweep of a sample step: the charge pass over every site's triangles and
// the per-chain finish (nmmc_sweep_measure's fused form on the HBM four-site path).
int launch_measure_fused_tail(Ctx& c, const int* d_chains, int n, int accumulate) {
    const MeasureShape ms = measure_shape(c);
    if ((size_t)n * measure_partials_per_chain(c) > c.partial_cap || (size_t)n * q4_meas_blocks(c) * 10 > c.mrows_cap)
        return set_error(NMMC_ERR_ARG, "fused measurement scratch not prepared");
    const float* sp = (const float*)c.d_spins;
    // sliding-row charge pass: strips of four sites (edge a multiple of 4, at most 256 strips
    // of a row per block), nseg row segments of R rows per block
    const int nstrip = c.m.hx / 2;
    if (c.charge_pass == 0 && c.m.hx % 2 == 0 && nstrip >= 1 && nstrip <= 256) {
        const int nseg = 256 / nstrip;
        const int R = std::min(16, (c.m.ly + nseg - 1) / nseg);
        const int nblk_slice = (c.m.ly + nseg * R - 1) / (nseg * R);
        const int nblk = nblk_slice * c.m.lz;
        if ((size_t)n * nblk * kNP <= c.partial_cap) {
            dim3 grid(nblk, n);
            if (c.periodic)
                k_charge_rows<true><<<grid, 256, 0, c.stream>>>(c.m, sp, d_chains, nstrip, nseg, R, nblk_slice,
                                                                c.d_partial);
            else
                k_charge_rows<false><<<grid, 256, 0, c.stream>>>(c.m, sp, d_chains, nstrip, nseg, R, nblk_slice,
                                                                 c.d_partial);
            const int nb = q4_meas_blocks(c);
            k_measure_finalize_fused<<<n, 256, 0, c.stream>>>(d_chains, c.d_partial, nblk, nblk_slice, c.m.lz,
                                                              c.d_mrows, nb, c.d_Hd, c.d_obs, c.d_q, c.d_acc,
                                                              accumulate);
            return cuda_check(cudaGetLastError(), "fused measure launch");
        }
    }
    dim3 grid(ms.nblk, n);
#define NMMC_QP(D, PER)                                                                                        \
    do {                                                                                                       \
        if (c.measure_sites == 4)                                                                              \
            k_measure_q4<D, PER, kDmiNone, 4, true><<<grid, 256, 0, c.stream>>>(c.m, sp, d_chains, ms.rows,   \
                                                                                ms.nblk_slice, c.d_partial);   \
        else                                                                                                   \
            k_measure_q4<D, PER, kDmiNone, 2, true><<<grid, 256, 0, c.stream>>>(c.m, sp, d_chains, ms.rows,   \
                                                                                ms.nblk_slice, c.d_partial);   \
    } while (0)
    if (c.dim == 3) { if (c.periodic) NMMC_QP(3, true); else NMMC_QP(3, false); }
    else { if (c.periodic) NMMC_QP(2, true); else NMMC_QP(2, false); }
#undef NMMC_QP
    const int nb = q4_meas_blocks(c);
    k_measure_finalize_fused<<<n, 256, 0, c.stream>>>(d_chains, c.d_partial, ms.nblk, ms.nblk_slice, c.m.lz,
                                                      c.d_mrows, nb, c.d_Hd, c.d_obs, c.d_q, c.d_acc, accumulate);
    return cuda_check(cudaGetLastError(), "fused measure launch");
}

// Measurement into caller-provided partial-sum scratch and caller-provided outputs, with the
// block split of launch_measure (the same sums in the same order). No allocation.
int launch_measure_into(Ctx& c, const int* d_chains, int n, double* scratch, size_t scratch_doubles,
                        double* obs, double* q) {
    if ((size_t)n * measure_partials_per_chain(c) > scratch_doubles)
        return set_error(NMMC_ERR_ARG, "%d chains need %zu scratch doubles, %zu given", n,
                         (size_t)n * measure_partials_per_chain(c), scratch_doubles);
    return measure_with(c, d_chains, n, scratch, obs, q, 0);
}

// ------------------------------------------------------------------------------------------
// dE probe: the sweep kernels' FP32 arithmetic on caller-chosen proposals.
// ------------------------------------------------------------------------------------------
template <int DIM, bool PERIODIC>
__global__ void k_delta_e(const DevModel m, const void* __restrict__ spins_v, const float4* __restrict__ bh,
                          int chain, const int32_t* __restrict__ sites, const float* __restrict__ trial,
                          int n, double* __restrict__ out) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int box = sites[t];
    const int x = box % m.edge;
    const int y = (box / m.edge) % m.edge;
    const int z = (DIM == 3) ? box / (m.edge * m.edge) : 0;
    const int colour = (x + y + z) & 1;
    const int i = (z * m.ly + y) * m.hx + (x >> 1);
    const size_t P = (size_t)m.nhalf_pad;
    const float4 p = bh[chain];
    constexpr int ND = 2 * DIM;
    if (m.ising) {
        const int8_t* own = (const int8_t*)spins_v + ((size_t)chain * 2 + colour) * P;
        const int8_t* oth = (const int8_t*)spins_v + ((size_t)chain * 2 + (colour ^ 1)) * P;
        float nb[ND];
#pragma unroll
        for (int k = 0; k < ND; ++k) {
            int j = nb_compact<PERIODIC>(m, x, y, z, k);
            nb[k] = (j >= 0) ? (float)oth[j] : 0.0f;
        }
        float h = ising_field<ND>(m, nb, p);
        out[t] = (double)(h * ((float)own[i] - trial[3 * t]));
    } else {
        const float* own = (const float*)spins_v + ((size_t)chain * 2 + colour) * 3 * P;
        const float* oth = (const float*)spins_v + ((size_t)chain * 2 + (colour ^ 1)) * 3 * P;
        float nx[ND], ny[ND], nz[ND];
#pragma unroll
        for (int k = 0; k < ND; ++k) {
            int j = nb_compact<PERIODIC>(m, x, y, z, k);
            nx[k] = j >= 0 ? oth[j] : 0.f;
            ny[k] = j >= 0 ? oth[P + j] : 0.f;
            nz[k] = j >= 0 ? oth[2 * P + j] : 0.f;
        }
        float hx, hy, hz;
        switch (m.dmi_kind) {
            case kDmiNone: heis_field<ND, kDmiNone>(m, nx, ny, nz, p, hx, hy, hz); break;
            case kDmiGeneral: heis_field<ND, kDmiGeneral>(m, nx, ny, nz, p, hx, hy, hz); break;
            case kDmiPairs: heis_field<ND, kDmiPairs>(m, nx, ny, nz, p, hx, hy, hz); break;
            default: heis_field<ND, kDmiAxial>(m, nx, ny, nz, p, hx, hy, hz); break;
        }
        out[t] = (double)heis_dE(hx, hy, hz, own[i], own[P + i], own[2 * P + i], trial[3 * t],
                                 trial[3 * t + 1], trial[3 * t + 2]);
    }
}

int launch_delta_e(Ctx& c, int chain, const int32_t* d_sites, const float* d_trial, int n, double* d_out) {
    int g = (n + 127) / 128;
    if (c.dim == 3) {
        if (c.periodic) k_delta_e<3, true><<<g, 128, 0, c.stream>>>(c.m, c.d_spins, c.d_bh, chain, d_sites, d_trial, n, d_out);
        else k_delta_e<3, false><<<g, 128, 0, c.stream>>>(c.m, c.d_spins, c.d_bh, chain, d_sites, d_trial, n, d_out);
    } else {
        if (c.periodic) k_delta_e<2, true><<<g, 128, 0, c.stream>>>(c.m, c.d_spins, c.d_bh, chain, d_sites, d_trial, n, d_out);
        else k_delta_e<2, false><<<g, 128, 0, c.stream>>>(c.m, c.d_spins, c.d_bh, chain, d_sites, d_trial, n, d_out);
    }
    return cuda_check(cudaGetLastError(), "k_delta_e");
}

// ------------------------------------------------------------------------------------------
// Sequential FP64 replay of a logged random-site chain (one thread). Arithmetic follows
// the reference's order exactly (records in file order; res_c = (H_c + Vsum_c) * Vdiff_c;
// dE = res_0 + res_1 + res_2) with every operation rounded separately, so it matches a
// host FP64 restatement built without floating-point contraction.
// ------------------------------------------------------------------------------------------
__global__ void k_to_fp64(const DevModel m, const void* __restrict__ spins_v, int chain, double* __restrict__ S) {
    long long box = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long nbox = (long long)m.edge * m.edge * m.lz;
    if (box >= nbox) return;
    int x = (int)(box % m.edge), y = (int)((box / m.edge) % m.edge), z = (int)(box / ((long long)m.edge * m.edge));
    int colour = (x + y + z) & 1;
    size_t i = (size_t)(z * m.ly + y) * m.hx + (x >> 1);
    size_t P = (size_t)m.nhalf_pad;
    if (m.ising) {
        S[3 * box] = (double)((const int8_t*)spins_v)[((size_t)chain * 2 + colour) * P + i];
        S[3 * box + 1] = S[3 * box + 2] = 0.0;
    } else {
        const float* pl = (const float*)spins_v + ((size_t)chain * 2 + colour) * 3 * P;
        S[3 * box] = pl[i];
        S[3 * box + 1] = pl[P + i];
        S[3 * box + 2] = pl[2 * P + i];
    }
}

__global__ void k_from_fp64(const DevModel m, void* __restrict__ spins_v, const uint8_t* __restrict__ mask,
                            int chain, const double* __restrict__ S) {
    long long box = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long nbox = (long long)m.edge * m.edge * m.lz;
    if (box >= nbox) return;
    int x = (int)(box % m.edge), y = (int)((box / m.edge) % m.edge), z = (int)(box / ((long long)m.edge * m.edge));
    int colour = (x + y + z) & 1;
    size_t i = (size_t)(z * m.ly + y) * m.hx + (x >> 1);
    size_t P = (size_t)m.nhalf_pad;
    if (mask && !mask[((size_t)chain * 2 + colour) * P + i]) return;
    if (m.ising) {
        ((int8_t*)spins_v)[((size_t)chain * 2 + colour) * P + i] = (int8_t)S[3 * box];
    } else {
        float* pl = (float*)spins_v + ((size_t)chain * 2 + colour) * 3 * P;
        pl[i] = (float)S[3 * box];
        pl[P + i] = (float)S[3 * box + 1];
        pl[2 * P + i] = (float)S[3 * box + 2];
    }
}

__global__ void k_replay(const DevModel m, const ReplayModel* __restrict__ rmp, double* __restrict__ S,
                         const uint8_t* __restrict__ mask, int chain, const nmmc_event* __restrict__ ev,
                         long long n, double beta, double H0, double H1, double H2,
                         uint8_t* __restrict__ acc_out, long long* __restrict__ first, int* __restrict__ flag) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const ReplayModel& rm = *rmp;
    const long long nbox = (long long)m.edge * m.edge * m.lz;
    const size_t P = (size_t)m.nhalf_pad;
    auto filled = [&](int x, int y, int z) -> bool {
        if (!mask) return x < m.edge;
        int colour = (x + y + z) & 1;
        return mask[((size_t)chain * 2 + colour) * P + (size_t)(z * m.ly + y) * m.hx + (x >> 1)] != 0;
    };
    const double H[3] = {H0, H1, H2};
    long long fm = -1;
    for (long long e = 0; e < n; ++e) {
        const int site = ev[e].site_box;
        if (site < 0 || site >= nbox) { *flag = 1; break; }
        const int x = site % m.edge, y = (site / m.edge) % m.edge, z = site / (m.edge * m.edge);
        if (!filled(x, y, z)) { *flag = 2; break; }
        double t[3] = {ev[e].trial[0], ev[e].trial[1], ev[e].trial[2]};
        double vdiff[3], vsum[3] = {0.0, 0.0, 0.0};
        for (int c = 0; c < 3; ++c) vdiff[c] = __dsub_rn(S[3 * site + c], t[c]);
        for (int r = 0; r < rm.n; ++r) {
            int q[3] = {x + rm.off[r][0], y + rm.off[r][1], z + (m.dim == 3 ? rm.off[r][2] : 0)};
            bool ok = true;
            for (int a = 0; a < m.dim; ++a) {
                if (m.periodic) q[a] = (m.edge + (q[a] % m.edge)) % m.edge;
                else if (q[a] < 0 || q[a] >= m.edge) ok = false;
            }
            if (!ok || !filled(q[0], q[1], q[2])) continue;
            const int nb = q[0] + m.edge * (q[1] + m.edge * q[2]);
            if (nb == site) continue;
            const double* sj = S + 3 * (size_t)nb;
            if (rm.useJ)
                for (int c = 0; c < 3; ++c) vsum[c] = __dadd_rn(vsum[c], __dmul_rn(rm.J[r], sj[c]));
            if (rm.useD) {
                const double* D = rm.D[r];
                double o[3];
                if (rm.dmi_sign == 0) {   // s_j x D (as the reference's dE)
                    o[0] = __dsub_rn(__dmul_rn(sj[1], D[2]), __dmul_rn(sj[2], D[1]));
                    o[1] = __dsub_rn(__dmul_rn(sj[2], D[0]), __dmul_rn(sj[0], D[2]));
                    o[2] = __dsub_rn(__dmul_rn(sj[0], D[1]), __dmul_rn(sj[1], D[0]));
                } else {                  // D x s_j
                    o[0] = __dsub_rn(__dmul_rn(D[1], sj[2]), __dmul_rn(D[2], sj[1]));
                    o[1] = __dsub_rn(__dmul_rn(D[2], sj[0]), __dmul_rn(D[0], sj[2]));
                    o[2] = __dsub_rn(__dmul_rn(D[0], sj[1]), __dmul_rn(D[1], sj[0]));
                }
                for (int c = 0; c < 3; ++c) vsum[c] = __dadd_rn(vsum[c], o[c]);
            }
        }
        double res[3];
        for (int c = 0; c < 3; ++c) res[c] = __dmul_rn(__dadd_rn(H[c], vsum[c]), vdiff[c]);
        const double dE = __dadd_rn(__dadd_rn(res[0], res[1]), res[2]);
        int acc;
        if (dE <= 0) acc = 1;
        else acc = (__dmul_rn(-dE, beta) > log(ev[e].u)) ? 1 : 0;
        if (acc)
            for (int c = 0; c < 3; ++c) S[3 * site + c] = t[c];
        acc_out[e] = (uint8_t)acc;
        if (fm < 0 && acc != ev[e].accepted) fm = e;
    }
    *first = fm;
}

int launch_replay(Ctx& c, int chain, const nmmc_event* d_ev, size_t n, uint8_t* d_acc, long long* d_first) {
    long long nbox = c.box_sites;
    int g = (int)((nbox + 255) / 256);
    k_to_fp64<<<g, 256, 0, c.stream>>>(c.m, c.d_spins, chain, c.d_replay);
    double beta = 1.0 / (c.k_b * c.T[chain]);
    double H[3] = {0, 0, 0};
    H[c.ising ? 0 : 2] = c.H[chain];
    k_replay<<<1, 1, 0, c.stream>>>(c.m, c.d_rm, c.d_replay, c.d_mask, chain, d_ev, (long long)n, beta,
                                    H[0], H[1], H[2], d_acc, d_first, c.d_flag);
    k_from_fp64<<<g, 256, 0, c.stream>>>(c.m, c.d_spins, c.d_mask, chain, c.d_replay);
    return cuda_check(cudaGetLastError(), "replay launch");
}

// ------------------------------------------------------------------------------------------
// Summed lattices (state::add_to_av, Old/lib/state.cpp:288-296): av[slot][box][c] += spin.
// ------------------------------------------------------------------------------------------
__global__ void k_add_av(const DevModel m, const void* __restrict__ spins_v, const int* __restrict__ list,
                         double* __restrict__ av) {
    const long long box = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long nbox = (long long)m.edge * m.edge * m.lz;
    if (box >= nbox) return;
    const int chain = list[blockIdx.y];
    const int x = (int)(box % m.edge), y = (int)((box / m.edge) % m.edge), z = (int)(box / ((long long)m.edge * m.edge));
    const int colour = (x + y + z) & 1;
    const size_t P = (size_t)m.nhalf_pad, i = (size_t)(z * m.ly + y) * m.hx + (x >> 1);
    double* a = av + ((size_t)blockIdx.y * nbox + box) * 3;
    if (m.ising) {
        a[0] += (double)((const int8_t*)spins_v)[((size_t)chain * 2 + colour) * P + i];
    } else {
        const float* pl = (const float*)spins_v + ((size_t)chain * 2 + colour) * 3 * P;
        a[0] += (double)pl[i];
        a[1] += (double)pl[P + i];
        a[2] += (double)pl[2 * P + i];
    }
}

int launch_add_av(Ctx& c) {
    if (c.av_chains.empty()) return NMMC_OK;
    dim3 grid((unsigned)((c.box_sites + 255) / 256), (unsigned)c.av_chains.size());
    k_add_av<<<grid, 256, 0, c.stream>>>(c.m, c.d_spins, c.d_av_list, c.d_av);
    return cuda_check(cudaGetLastError(), "k_add_av");
}

// ------------------------------------------------------------------------------------------
// Random start (field_type::all_rand, Old/lib/field_type.cpp:197-204)
// ------------------------------------------------------------------------------------------
__global__ void k_init_spins(const DevModel m, void* __restrict__ spins_v, const uint8_t* __restrict__ mask) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int chain = blockIdx.y;
    const int colour = blockIdx.z;
    const size_t P = (size_t)m.nhalf_pad;
    if (i >= m.nhalf_pad) return;
    bool fill = false;
    int x = 0, y = 0, z = 0;
    if (i < m.nhalf) {
        int row = i / m.hx, h = i - row * m.hx;
        z = (m.dim == 3) ? row / m.ly : 0;
        y = row - z * m.ly;
        x = 2 * h + ((y + z + colour) & 1);
        fill = mask ? mask[((size_t)chain * 2 + colour) * P + i] != 0 : (x < m.edge);
    }
    const uint32_t box = (uint32_t)(x + m.edge * (y + m.edge * z));
    nmmc_u4 r = nmmc_philox(box, 0u, NMMC_STREAM_INIT << 28, (uint32_t)chain, m.key0, m.key1);
    if (m.ising) {
        int8_t v = fill ? ((r.x >> 31) ? 1 : -1) : 0;
        ((int8_t*)spins_v)[((size_t)chain * 2 + colour) * P + i] = v;
    } else {
        float tx = 0, ty = 0, tz = 0;
        if (fill) {
            tz = fmaf(2.0f, nmmc_u01f(r.x), -1.0f);
            float sp, cp;
            sincospif(fmaf(2.0f, nmmc_u01f(r.y), -1.0f), &sp, &cp);
            float rxy = sqrtf(fmaxf(0.0f, 1.0f - tz * tz));
            tx = rxy * cp;
            ty = rxy * sp;
        }
        float* pl = (float*)spins_v + ((size_t)chain * 2 + colour) * 3 * P;
        pl[i] = tx;
        pl[P + i] = ty;
        pl[2 * P + i] = tz;
    }
}

int launch_init_spins(Ctx& c) {
    dim3 grid((c.m.nhalf_pad + 255) / 256, c.nchains, 2);
    k_init_spins<<<grid, 256, 0, c.stream>>>(c.m, c.d_spins, c.d_mask);
    return cuda_check(cudaGetLastError(), "k_init_spins");
}

}  // namespace nmmc
