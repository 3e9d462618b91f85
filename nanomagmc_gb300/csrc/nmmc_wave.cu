// Wavefront sweeps: both colours of a checkerboard sweep in one pass over the lattice.
//
// A sweep of state::equil (Old/lib/state.cpp:171-203) on the checkerboard is colour 0 over
// every site, then colour 1 over every site. A colour-0 update at plane z reads colour 1 at
// planes z-1, z, z+1 (old values); a colour-1 update at plane z reads colour 0 at the same
// planes (new values). So one CTA that marches along z can update colour 0 of plane t and
// colour 1 of plane t-2 in the same step (the latter's colour-0 neighbours, planes t-3 .. t-1,
// are all new by then): every site gets the same inputs and the same Philox counter as in the
// two half-sweeps, hence the same chain bit for bit, while every spin is read from HBM once
// and written once per sweep (24 B per site and sweep instead of 72 B for two streaming
// half-sweeps). On 40 chains of 128^3 it measured 1.26e11 updates/s against 1.53e11 for the
// half-sweeps (the per-step barrier and the dependent update chain, not DRAM, bound both), so
// it is opt-in (NMMC_OPT_WAVE).
//
// The sweep is out of place: it reads `src` and writes `dst`, so no CTA ever reads a value
// another CTA writes in the same launch. A CTA owns tiles of `rows` rows (y) of one chain over
// a run of z-planes; the colour-0 values it needs beyond its own rows (one row either side)
// and beyond its z-run (one plane either side) it computes again itself from `src` — the same
// values the owning CTA computes — and keeps the new colour-0 rows of the last planes in a
// shared-memory ring of four slots. Work is split evenly: the launch's (chain, tile, plane)
// units are cut into one contiguous run per CTA (a run may cross into the next tile or chain).
#include <algorithm>

#include "nmmc_kernels.cuh"

namespace nmmc {

constexpr int kWaveSlots = 4;
constexpr int kWaveMaxThreads = 256;

__device__ __forceinline__ float wel(const float4& v, int k) {
    return k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w));
}

// Four consecutive same-colour sites of one row (x = 2 (h0 + k) + xp), their neighbours given
// as the other colour's rows: `same` the same row, `ex` the x-neighbour outside the quad,
// yp/ym and zp/zm the rows at y +- 1 and z +- 1 (zero where a neighbour is missing). The
// arithmetic and the draw order are those of the four-site half-sweep (q4_quad), so the
// results are the same.
template <int DK, bool PERIODIC>
__device__ __forceinline__ void wave_quad(const DevModel& m, const float4 (&s)[3], const float4 (&same)[3],
                                          const float (&ex)[3], const float4 (&yp)[3], const float4 (&ym)[3],
                                          const float4 (&zp)[3], const float4 (&zm)[3], int xp, int h0,
                                          uint32_t boxrow, unsigned long long sw, int chain, float4 p,
                                          float (&out)[3][4]) {
    constexpr int ND = 6;
    nmmc_u4 rnext = sweep_draw<true>(m, boxrow + (uint32_t)(2 * h0 + xp), sw, (uint32_t)chain);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        float nx[ND], ny[ND], nz[ND];
        float* nn[3] = {nx, ny, nz};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float sm = wel(same[c], k);
            const float sh = xp ? (k < 3 ? wel(same[c], k + 1) : ex[c]) : (k > 0 ? wel(same[c], k - 1) : ex[c]);
            float plusx = xp ? sh : sm, minusx = xp ? sm : sh;
            if (!PERIODIC) {
                const int x = 2 * (h0 + k) + xp;
                if (x + 1 >= m.edge) plusx = 0.0f;
                if (x == 0) minusx = 0.0f;
            }
            nn[c][0] = plusx;
            nn[c][1] = minusx;
            nn[c][2] = wel(yp[c], k);
            nn[c][3] = wel(ym[c], k);
            nn[c][4] = wel(zp[c], k);
            nn[c][5] = wel(zm[c], k);
        }
        const float sx = wel(s[0], k), sy = wel(s[1], k), sz = wel(s[2], k);
        const nmmc_u4 r = rnext;
        if (k < 3) rnext = sweep_draw<true>(m, boxrow + (uint32_t)(2 * (h0 + k + 1) + xp), sw, (uint32_t)chain);
        float hx, hy, hz, tx, ty, tz;
        heis_field<ND, DK>(m, nx, ny, nz, p, hx, hy, hz);
        const bool acc = heis_try(hx, hy, hz, sx, sy, sz, p, r, tx, ty, tz);
        out[0][k] = acc ? tx : sx;
        out[1][k] = acc ? ty : sy;
        out[2][k] = acc ? tz : sz;
    }
}

// x-neighbour outside a quad: compact index h0 - 1 (xp = 0) or h0 + 4 (xp = 1), wrapped on
// periodic lattices; -1 when it falls off an open edge.
template <bool PERIODIC>
__device__ __forceinline__ int wave_hx_out(const DevModel& m, int h0, int xp) {
    int h = xp ? h0 + 4 : h0 - 1;
    if (PERIODIC) return (h < 0) ? m.hx - 1 : (h >= m.hx ? 0 : h);
    return (h >= 0 && h < m.hx) ? h : -1;
}

// Colour-0 quad at (plane z, row y): its old spins and the old colour-1 neighbours from src.
template <int DK, bool PERIODIC>
__device__ __forceinline__ void wave_c0_quad(const DevModel& m, const float* __restrict__ s0,
                                             const float* __restrict__ s1, size_t P, int z, int y, int h0,
                                             unsigned long long sw, int chain, float4 p, float (&out)[3][4]) {
    const int hx = m.hx, ly = m.ly, lz = m.lz;
    const int xp = (y + z) & 1;
    const int rb = (z * ly + y) * hx + h0;
    float4 s[3], same[3], yp[3], ym[3], zp[3], zm[3];
    float ex[3];
    const float4 vz = {};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        s[c] = __ldg(reinterpret_cast<const float4*>(s0 + c * P + rb));
        same[c] = __ldg(reinterpret_cast<const float4*>(s1 + c * P + rb));
    }
    const int hxo = wave_hx_out<PERIODIC>(m, h0, xp);
#pragma unroll
    for (int c = 0; c < 3; ++c) ex[c] = hxo >= 0 ? __ldg(s1 + c * P + (z * ly + y) * hx + hxo) : 0.0f;
    int yu = y + 1, yd = y - 1, zu = z + 1, zd = z - 1;
    bool okU = true, okD = true, oU = true, oD = true;
    if (PERIODIC) {
        yu = (yu == ly) ? 0 : yu;
        yd = (yd < 0) ? ly - 1 : yd;
        zu = (zu == lz) ? 0 : zu;
        zd = (zd < 0) ? lz - 1 : zd;
    } else {
        okU = yu < ly;
        okD = yd >= 0;
        oU = zu < lz;
        oD = zd >= 0;
    }
    const int ru = (z * ly + yu) * hx + h0, rd = (z * ly + yd) * hx + h0;
    const int rzu = (zu * ly + y) * hx + h0, rzd = (zd * ly + y) * hx + h0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        yp[c] = okU ? __ldg(reinterpret_cast<const float4*>(s1 + c * P + ru)) : vz;
        ym[c] = okD ? __ldg(reinterpret_cast<const float4*>(s1 + c * P + rd)) : vz;
        zp[c] = oU ? __ldg(reinterpret_cast<const float4*>(s1 + c * P + rzu)) : vz;
        zm[c] = oD ? __ldg(reinterpret_cast<const float4*>(s1 + c * P + rzd)) : vz;
    }
    const uint32_t boxrow = (uint32_t)(m.edge * (y + m.edge * z));
    wave_quad<DK, PERIODIC>(m, s, same, ex, yp, ym, zp, zm, xp, h0, boxrow, sw, chain, p, out);
}

// One launch = one sweep of the listed chains, src -> dst. A tile is the rows [ys, ye) of one
// chain; the CTA has (rmax + 2) x (sites per row / 4) threads, rmax >= ye - ys. Each step t of
// a run [za, zb) of planes is one phase: thread row r updates the colour-0 quad of row
// ys - 1 + r at plane t (rows ys-1 .. ye, the outer two computed again from src) into ring slot
// t & 3, and the colour-1 quad of row ys + r at plane t - 2, whose colour-0 neighbours (planes
// t-3 .. t-1) the ring holds from the previous steps; one barrier ends the step. The ring:
// [slot][component][rmax + 2 rows][hx] floats; ring row rr holds row ys - 1 + rr.
template <int DK, bool PERIODIC>
__global__ void __launch_bounds__(kWaveMaxThreads, 2)
k_heis_wave(const DevModel m, const float* __restrict__ src, float* __restrict__ dst,
            const float4* __restrict__ bh, const unsigned long long* __restrict__ sweep,
            const int* __restrict__ chains, int rmax, int ntile, unsigned sweep_off, long long units) {
    extern __shared__ float4 wave_ring4[];
    float* ring = reinterpret_cast<float*>(wave_ring4);
    const int hx = m.hx, qpr = hx >> 2, lz = m.lz, ly = m.ly;
    const int plane_f = (rmax + 2) * hx;   // floats of one component of one slot
    const int slot_f = 3 * plane_f;
    const size_t P = (size_t)m.nhalf_pad;
    const int tid = threadIdx.x;
    const int tr = tid / qpr, h0 = (tid - tr * qpr) * 4;
    const long long w0 = units * blockIdx.x / gridDim.x, w1 = units * (blockIdx.x + 1) / gridDim.x;

    for (long long w = w0; w < w1;) {
        const long long col = w / lz;
        const int za = (int)(w - col * lz);
        const int zb = (int)min((long long)lz, (long long)za + (w1 - w));
        w += zb - za;
        const int ci = (int)(col / ntile), ty = (int)(col - (long long)ci * ntile);
        const int chain = chains[ci];
        const int ys = ty * ly / ntile, ye = (ty + 1) * ly / ntile;
        const float4 p = bh[chain];
        const unsigned long long sw = sweep[chain] + sweep_off;
        const float* s0 = src + (size_t)chain * 6 * P;   // colour 0: 3 component planes
        const float* s1 = s0 + 3 * P;                     // colour 1
        float* d0 = dst + (size_t)chain * 6 * P;
        float* d1 = d0 + 3 * P;
        // this thread's colour-0 row (ring row tr) and colour-1 row
        int y0r = ys - 1 + tr;
        bool c0_row = tr < ye - ys + 2;
        if (PERIODIC) y0r = (y0r < 0) ? y0r + ly : (y0r >= ly ? y0r - ly : y0r);
        else c0_row = c0_row && y0r >= 0 && y0r < ly;
        const bool c0_in_ring = tr < ye - ys + 2;
        const bool c0_own = tr >= 1 && tr <= ye - ys;
        const int y1r = ys + tr;
        const bool c1_row = y1r < ye;

        for (int t = za - 1; t <= zb + 1; ++t) {
            // colour 1 of plane t - 2 from the ring (slots of planes t-3, t-2, t-1)
            const int zc = t - 2;
            if (c1_row && zc >= za && zc < zb) {
                const int rr = tr + 1;
                const int xp = (y1r + zc + 1) & 1;
                const int rb = (zc * ly + y1r) * hx + h0;
                const float* sc = ring + ((t - 2) & 3) * slot_f;
                const float* su = ring + ((t - 1) & 3) * slot_f;
                const float* sd = ring + ((t - 3) & 3) * slot_f;
                float4 s[3], same[3], yp[3], ym[3], zp[3], zm[3];
                float ex[3];
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    s[c] = __ldg(reinterpret_cast<const float4*>(s1 + c * P + rb));
                    same[c] = *reinterpret_cast<const float4*>(sc + c * plane_f + rr * hx + h0);
                    yp[c] = *reinterpret_cast<const float4*>(sc + c * plane_f + (rr + 1) * hx + h0);
                    ym[c] = *reinterpret_cast<const float4*>(sc + c * plane_f + (rr - 1) * hx + h0);
                    zp[c] = *reinterpret_cast<const float4*>(su + c * plane_f + rr * hx + h0);
                    zm[c] = *reinterpret_cast<const float4*>(sd + c * plane_f + rr * hx + h0);
                }
                const int hxo = wave_hx_out<PERIODIC>(m, h0, xp);
#pragma unroll
                for (int c = 0; c < 3; ++c) ex[c] = hxo >= 0 ? sc[c * plane_f + rr * hx + hxo] : 0.0f;
                const uint32_t boxrow = (uint32_t)(m.edge * (y1r + m.edge * zc));
                float out[3][4];
                wave_quad<DK, PERIODIC>(m, s, same, ex, yp, ym, zp, zm, xp, h0, boxrow, sw, chain, p, out);
#pragma unroll
                for (int c = 0; c < 3; ++c)
                    *reinterpret_cast<float4*>(d1 + c * P + rb) = make_float4(out[c][0], out[c][1], out[c][2], out[c][3]);
            }
            // colour 0 of plane t into ring slot t & 3 (zero where the plane or row is missing)
            if (c0_in_ring && t <= zb) {
                int z = t;
                bool ok = c0_row;
                if (PERIODIC) z = (t < 0) ? t + lz : (t >= lz ? t - lz : t);
                else ok = ok && t >= 0 && t < lz;
                float out[3][4];
                if (ok) {
                    wave_c0_quad<DK, PERIODIC>(m, s0, s1, P, z, y0r, h0, sw, chain, p, out);
                    if (c0_own && t >= za && t < zb) {
                        const int rb = (z * ly + y0r) * hx + h0;
#pragma unroll
                        for (int c = 0; c < 3; ++c)
                            *reinterpret_cast<float4*>(d0 + c * P + rb) =
                                make_float4(out[c][0], out[c][1], out[c][2], out[c][3]);
                    }
                } else {
#pragma unroll
                    for (int c = 0; c < 3; ++c) out[c][0] = out[c][1] = out[c][2] = out[c][3] = 0.0f;
                }
                float* slot = ring + (t & 3) * slot_f;
#pragma unroll
                for (int c = 0; c < 3; ++c)
                    *reinterpret_cast<float4*>(slot + c * plane_f + tr * hx + h0) =
                        make_float4(out[c][0], out[c][1], out[c][2], out[c][3]);
            }
            __syncthreads();
        }
    }
}

// Tile shape of the wavefront sweep on this lattice (false: the lattice is not covered):
// 3-D unmasked Heisenberg lattices with the checkerboard's axis tables and rows of a multiple
// of 4 sites per colour. rmax + 2 thread rows of (sites per row / 4) threads, at most 256;
// ntile tiles of ly / ntile rows (rounded) per plane.
static bool wave_shape(const Ctx& c, int& rmax, int& ntile) {
    if (c.ising || c.masked || c.m.general || c.dim != 3 || (c.m.hx % 4) != 0) return false;
    const int qpr = c.m.hx / 4;
    const int trows = std::min(kWaveMaxThreads / qpr, c.m.ly + 2);
    if (trows < 3) return false;
    ntile = (c.m.ly + trows - 3) / (trows - 2);
    rmax = (c.m.ly + ntile - 1) / ntile;
    return true;
}

int wave_rows(const Ctx& c) {
    int rmax = 0, ntile = 0;
    return wave_shape(c, rmax, ntile) ? rmax : 0;
}

static size_t wave_smem(const Ctx& c, int rmax) {
    return (size_t)kWaveSlots * 3 * (rmax + 2) * c.m.hx * sizeof(float);
}

template <int DK, bool PERIODIC>
static int wave_launch_t(Ctx& c, const float* src, float* dst, const int* d_chains, int n, unsigned off) {
    int rmax = 0, ntile = 0;
    if (!wave_shape(c, rmax, ntile)) return set_error(NMMC_ERR_UNSUPPORTED, "lattice not covered by the wave sweep");
    const int threads = (rmax + 2) * (c.m.hx / 4);
    const size_t smem = wave_smem(c, rmax);
    auto kern = k_heis_wave<DK, PERIODIC>;
    int& per_sm = c.wave_per_sm[DK * 2 + (PERIODIC ? 1 : 0)];
    if (per_sm == 0) {   // once per kernel and context (the tile shape is fixed by the lattice)
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return cuda_check(e, "wave sweep shared memory");
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem);
        if (e != cudaSuccess) return cuda_check(e, "wave sweep occupancy");
        if (per_sm < 1) {
            per_sm = 0;
            return set_error(NMMC_ERR_CUDA, "wave sweep does not fit on an SM");
        }
    }
    const long long units = (long long)n * ntile * c.m.lz;
    // runs of at least 8 planes (each run recomputes two planes of colour 0)
    long long grid = std::min<long long>((long long)per_sm * c.sm_count, (units + 7) / 8);
    if (grid < 1) grid = 1;
    kern<<<(unsigned)grid, threads, smem, c.stream>>>(c.m, src, dst, c.d_bh, c.d_sweep, d_chains, rmax, ntile, off,
                                                      units);
    return cuda_check(cudaGetLastError(), "k_heis_wave");
}

// One wavefront sweep of the listed chains with Philox sweep offset `off`, src -> dst.
int launch_wave_sweep(Ctx& c, const float* src, float* dst, const int* d_chains, int n, unsigned off) {
    const bool per = c.periodic;
    switch (c.m.dmi_kind) {
        case kDmiNone: return per ? wave_launch_t<kDmiNone, true>(c, src, dst, d_chains, n, off)
                                  : wave_launch_t<kDmiNone, false>(c, src, dst, d_chains, n, off);
        case kDmiGeneral: return per ? wave_launch_t<kDmiGeneral, true>(c, src, dst, d_chains, n, off)
                                     : wave_launch_t<kDmiGeneral, false>(c, src, dst, d_chains, n, off);
        case kDmiPairs: return per ? wave_launch_t<kDmiPairs, true>(c, src, dst, d_chains, n, off)
                                   : wave_launch_t<kDmiPairs, false>(c, src, dst, d_chains, n, off);
        default: return per ? wave_launch_t<kDmiAxial, true>(c, src, dst, d_chains, n, off)
                            : wave_launch_t<kDmiAxial, false>(c, src, dst, d_chains, n, off);
    }
}

}  // namespace nmmc
