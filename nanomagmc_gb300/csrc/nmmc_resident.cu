// Shared-memory resident checkerboard sweeps for lattices that fit on chip: the 2-D runs and
// the batched Weibull nanoparticles. One persistent CTA owns a "bin" of whole chains: it
// loads their filled sites into shared memory once, runs all requested sweeps there with a
// __syncthreads between colours, and writes the spins back once. This replaces the
// reference's MPI split over lattices, temperatures and fields (Old/lib/main.cpp:104-275,
// Old/lib/protocol.cpp:97-131): every chain of the batch is a slot in some bin.
//
// Sites are stored compactly (only filled sites, colour 0 first, chain by chain), each with a
// 16-byte record of bin-local neighbour indices, box index and slot, so uneven particle sizes
// cost only their own sites and a site costs one vector load per sweep. Bins are packed
// longest-processing-time first; the bin count and CTA width are chosen by timing candidates
// on the live context (autotune) and cached per (model, sizes, GPU).
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>

#include <algorithm>
#include <fstream>
#include <numeric>
#include <sstream>

#include "nmmc_kernels.cuh"

namespace nmmc {

constexpr int kMaxSlots = 64;                 // chains per bin (6 bits of the record)
constexpr uint16_t kNoNb = 0xFFFF;            // host-side marker before the zero site is known
constexpr uint32_t kBoxBits = 26;             // record.w = box | slot << 26
constexpr uint32_t kBoxMask = (1u << kBoxBits) - 1;

// Per-site record: x = j0 | j1 << 16, y = j2 | j3 << 16, z = j4 | j5 << 16 (3-D), with j_k the
// bin-local index of the neighbour in stencil direction k (+x,-x,+y,-y,+z,-z); an absent
// neighbour (open edge, outside the particle) points at the bin's zero site, index cap, whose
// spin is held at 0. w = logical box index (the RNG counter) | chain slot << 26.
__device__ __forceinline__ int rec_nb(const uint4& r, int k) {
    const uint32_t w = (k < 2) ? r.x : ((k < 4) ? r.y : r.z);
    return (k & 1) ? (int)(w >> 16) : (int)(w & 0xFFFFu);
}

// Outputs of the fused measurement (MEASURE variants of k_resident).
struct FusedMeasure {
    double* obs;              // per list position: NMMC_OBS_N doubles
    double* q;                // per list position: the slice's topological charge
    double* acc;              // per chain accumulators
    const double* Hd;         // per chain FP64 field
    const int* pos;           // chain -> list position; nullptr: the list is every chain in order
    const int* slot_red;      // per bin-chain entry: bin-local first colour-0 site
    const int* slot_black;    // per bin-chain entry: bin-local first colour-1 site
    int accumulate;
};

// Per-site terms of the observables of a 2-D site held in shared memory (the same terms as
// the global measurement kernels, Old/lib/thermodynamics.cpp:71-198): energy density
// s . sum_k (J_k s_k + De_k x s_k), M, subM(0), sub4M and the two solid-angle triangles
// (i, i-x, i+y), (i, i+x, i-y), which use the unwrapped adjacency unless periodic_q.
// Ising spins are one float per site (sx), Heisenberg spins one float4 (x, y, z, 0) per site (s4).
template <bool ISING>
__device__ __forceinline__ void resident_site_terms(const DevModel& m, int t, bool red, const float* sx,
                                                    const float4* s4, const uint4 r4, int zero, float* acc) {
    float s0, s1 = 0.0f, s2 = 0.0f;
    if (ISING) {
        s0 = sx[t];
    } else {
        const float4 v = s4[t];
        s0 = v.x;
        s1 = v.y;
        s2 = v.z;
    }
    float f0 = 0.f, f1 = 0.f, f2 = 0.f;
#pragma unroll
    for (int d = 0; d < 4; ++d) {   // absent neighbours read the zero site
        const int j = rec_nb(r4, d);
        const float J = m.J[d];
        float n0, n1 = 0.0f, n2 = 0.0f;
        if (ISING) {
            n0 = sx[j];
        } else {
            const float4 v = s4[j];
            n0 = v.x;
            n1 = v.y;
            n2 = v.z;
        }
        f0 = fmaf(J, n0, f0);
        if (!ISING) {
            f1 = fmaf(J, n1, f1);
            f2 = fmaf(J, n2, f2);
            if (m.has_dmi) {   // De x s_j
                f0 = fmaf(m.De[d][1], n2, fmaf(-m.De[d][2], n1, f0));
                f1 = fmaf(m.De[d][2], n0, fmaf(-m.De[d][0], n2, f1));
                f2 = fmaf(m.De[d][0], n1, fmaf(-m.De[d][1], n0, f2));
            }
        }
    }
    acc[0] = fmaf(s0, f0, fmaf(s1, f1, fmaf(s2, f2, acc[0])));
    acc[1] += s0;
    acc[2] += s1;
    acc[3] += s2;
    if (red) {   // subM(0): (sum of coordinates) % 2 == 0
        acc[4] += s0;
        acc[5] += s1;
        acc[6] += s2;
    }
    const int box = (int)(r4.w & kBoxMask);
    const int y = box / m.edge, x = box - y * m.edge;
    {   // sub4M (thermodynamics.cpp:138-163), C truncating remainders; z = 0
        const int possum = x + y, posdiff = -x + y + (m.edge - m.edge % 4);
        if (possum % 4 == 0 && posdiff % 4 == 0) {
            acc[7] += s0;
            acc[8] += s1;
            acc[9] += s2;
        }
    }
    if (!ISING) {
        const int j0 = rec_nb(r4, 0), j1 = rec_nb(r4, 1), j2 = rec_nb(r4, 2), j3 = rec_nb(r4, 3);
        const bool pq = m.periodic && m.periodic_q;
        const bool qxp = j0 != zero && (x + 1 < m.edge || pq), qxm = j1 != zero && (x >= 1 || pq);
        const bool qyp = j2 != zero && (y + 1 < m.edge || pq), qym = j3 != zero && (y >= 1 || pq);
        if (qxm && qyp) {
            const float4 a = s4[j1], b = s4[j2];
            acc[10] += solid_angle_f(s0, s1, s2, a.x, a.y, a.z, b.x, b.y, b.z);
        }
        if (qxp && qym) {
            const float4 a = s4[j0], b = s4[j3];
            acc[10] += solid_angle_f(s0, s1, s2, a.x, a.y, a.z, b.x, b.y, b.z);
        }
    }
}

// Register cap of every k_resident variant; 0 (default): the compiler's choice under
// __launch_bounds__(1024), about 44 registers for the sweeps and 58 with the observables,
// i.e. one 1024-thread block per SM. At 40 no Heisenberg variant spills and two 768-thread
// blocks fit per SM, but on GB300 that measured 3-4% slower on the batched-grain and 2-D
// workloads (the autotuner still chose one block of 1024 threads per SM).
#ifndef NMMC_RESIDENT_MAXNREG
#define NMMC_RESIDENT_MAXNREG 0
#endif
#if NMMC_RESIDENT_MAXNREG > 0
#define NMMC_RESIDENT_BOUNDS __maxnreg__(NMMC_RESIDENT_MAXNREG)
#else
#define NMMC_RESIDENT_BOUNDS __launch_bounds__(1024)
#endif

// Kernel arguments (one struct, so every instantiation has the same signature).
struct ResidentArgs {
    void* spins;
    const float4* bh;
    unsigned long long* sweep;
    const uint8_t* active;
    const uint32_t* goff;     // per site: offset of component 0 in the spin array
    const uint4* rec;         // per site record (rec_nb)
    const int* bin_begin;     // nbins+1 site offsets
    const int* bin_nred;      // colour-0 sites of each bin
    const int* bin_cbeg;      // nbins+1 offsets into bin_chains
    const int* bin_chains;
    int nbins, cap, nsweeps;
    const uint4* draws;       // drawn-ahead variant: [sweep of this launch][site] Philox words
    long long draw_row;       // sites per sweep row of draws
};

// Byte offset of the drawn-ahead variant's two per-sweep buffers of Philox words in the
// dynamic shared memory: after the spins (cap + 1 sites of `site_bytes`), 16-byte aligned.
__host__ __device__ constexpr size_t draw_smem_offset(int cap, int site_bytes) {
    return ((size_t)(cap + 1) * site_bytes + 15) & ~(size_t)15;
}

// 16-byte global -> shared copies that complete asynchronously (cp.async, grouped per thread).
__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gmem_src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// Drawn-ahead variant, first kernel: the Philox words of sweeps [0, nsweeps) of this launch for
// every site of the resident tables, row k = the chain's sweep counter + k: exactly the words
// sweep_draw gives the resident kernel's update of that site and sweep. Sites of chains that
// this call does not sweep are skipped (their rows are never read). Runs on every SM, so the
// generator's instructions leave the resident kernel's dependent path.
__global__ void __launch_bounds__(256) k_predraw(const DevModel m, const uint4* __restrict__ rec,
                                                 const int* __restrict__ site_chain,
                                                 const uint8_t* __restrict__ active,
                                                 const unsigned long long* __restrict__ sweep, uint4* draws,
                                                 int nsites, int nsweeps) {
    const long long total = (long long)nsites * nsweeps;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(i / nsites), t = (int)(i - (long long)k * nsites);
        const int ch = site_chain[t];
        if (!active[ch]) continue;
        const nmmc_u4 r = sweep_draw(m, rec[t].w & kBoxMask, sweep[ch] + (unsigned)k, (uint32_t)ch);
        draws[i] = make_uint4(r.x, r.y, r.z, r.w);
    }
}

// MEASURE: after the last sweep, the bin's observables are computed from the spins still in
// shared memory and written straight to the outputs (no partial-sum pass over HBM). Each
// chain slot is summed by a fixed group of warps: FP32 per thread and per warp, FP64 across
// the group's warps in a fixed order, so results are reproducible run to run.
//
// PRE (drawn-ahead variant): the Philox words of every site and sweep come from k_predraw's
// rows instead of sweep_draw. Each thread copies the words of the sites it updates (the same
// sites every sweep) for sweep sw + 1 into one of two shared buffers by cp.async while it
// updates sweep sw, and waits for its own copies only; the update itself is unchanged.
template <int DIM, int DK, bool ISING, bool MEASURE, bool PRE>
__global__ void NMMC_RESIDENT_BOUNDS
k_resident(const DevModel m, const ResidentArgs a, const FusedMeasure fm) {
    static_assert(!MEASURE || DIM == 2, "the fused measurement covers one z-slice");
    extern __shared__ __align__(16) float sm[];
    __shared__ float4 sp[kMaxSlots];                 // (beta, H) of each slot
    __shared__ unsigned long long ssw[kMaxSlots];    // sweep counter of each slot
    __shared__ int sch[kMaxSlots];                   // chain of each slot; -1 - chain if inactive
    constexpr int ND = 2 * DIM;
    const size_t P = (size_t)m.nhalf_pad;
    const int cap = a.cap;   // the zero site
    float* sx = sm;                                // Ising: one float per site
    float4* s4 = reinterpret_cast<float4*>(sm);    // Heisenberg: (x, y, z, 0) per site, one 16-byte access
    // PRE: two buffers of cap words each (sweep parity)
    uint4* dbuf = reinterpret_cast<uint4*>(reinterpret_cast<char*>(sm) + draw_smem_offset(cap, ISING ? 4 : 16));
    for (int b = blockIdx.x; b < a.nbins; b += gridDim.x) {
        const int s0 = a.bin_begin[b], n = a.bin_begin[b + 1] - s0, nred = a.bin_nred[b];
        const int c0 = a.bin_cbeg[b], nslot = a.bin_cbeg[b + 1] - c0;
        const uint4* rec = a.rec + s0;
        // copies of sweep k's words of this thread's sites (both colours) into buffer k & 1
        auto fetch_draws = [&](int k) {
            uint4* dst = dbuf + (k & 1) * cap;
            const uint4* src = a.draws + (long long)k * a.draw_row + s0;
            for (int t = threadIdx.x; t < nred; t += blockDim.x) cp_async16(dst + t, src + t);
            for (int t = nred + threadIdx.x; t < n; t += blockDim.x) cp_async16(dst + t, src + t);
            cp_async_commit();
        };
        for (int t = threadIdx.x; t < nslot; t += blockDim.x) {
            const int ch = a.bin_chains[c0 + t];
            sch[t] = a.active[ch] ? ch : -1 - ch;
            sp[t] = a.bh[ch];
            ssw[t] = a.sweep[ch];
        }
        for (int t = threadIdx.x; t < n; t += blockDim.x) {
            const uint32_t off = a.goff[s0 + t];
            if (ISING) {
                sx[t] = (float)((const int8_t*)a.spins)[off];
            } else {
                const float* f = (const float*)a.spins;
                s4[t] = make_float4(f[off], f[off + P], f[off + 2 * P], 0.0f);
            }
        }
        if (threadIdx.x == 0) {
            if (ISING) sx[cap] = 0.0f;
            else s4[cap] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
        // this thread's first site record of each colour: the same in every sweep, so it is
        // loaded once and not at the start of every half-sweep (the later sites' records are
        // loaded one site ahead in the loop)
        const uint4 rfirst0 = ((int)threadIdx.x < nred) ? rec[threadIdx.x] : make_uint4(0, 0, 0, 0);
        const uint4 rfirst1 = (nred + (int)threadIdx.x < n) ? rec[nred + threadIdx.x] : make_uint4(0, 0, 0, 0);
        if (PRE && a.nsweeps > 0) fetch_draws(0);
        __syncthreads();
        for (int sw = 0; sw < a.nsweeps; ++sw) {
            if (PRE) {
                // buffer (sw + 1) & 1 was last read in sweep sw - 1, before this thread's
                // __syncthreads of that sweep; the wait covers this thread's copies of sweep sw
                if (sw + 1 < a.nsweeps) {
                    fetch_draws(sw + 1);
                    cp_async_wait<1>();
                } else {
                    cp_async_wait<0>();
                }
            }
            const uint4* drow = dbuf + (sw & 1) * cap;
            for (int colour = 0; colour < 2; ++colour) {
                const int lo = colour ? nred : 0, hi = colour ? n : nred;
                int t = lo + threadIdx.x;
                uint4 rn = colour ? rfirst1 : rfirst0;
                for (; t < hi; t += blockDim.x) {
                    const uint4 r4 = rn;   // this site's record; the next one is loaded ahead
                    if (t + (int)blockDim.x < hi) rn = rec[t + blockDim.x];
                    const int sl = (int)(r4.w >> kBoxBits);
                    const int ch = sch[sl];
                    if (ch < 0) continue;
                    nmmc_u4 r;
                    if (PRE) {
                        const uint4 d = drow[t];
                        r = nmmc_u4{d.x, d.y, d.z, d.w};
                    } else {
                        r = sweep_draw(m, r4.w & kBoxMask, ssw[sl] + (unsigned)sw, (uint32_t)ch);
                    }
                    if (ISING) {
                        float nb[ND];
#pragma unroll
                        for (int k = 0; k < ND; ++k) nb[k] = sx[rec_nb(r4, k)];
                        float tnew;
                        if (ising_attempt<ND>(m, sx[t], nb, sp[sl], r, tnew)) sx[t] = tnew;
                    } else {
                        float nx[ND], ny[ND], nz[ND];
#pragma unroll
                        for (int k = 0; k < ND; ++k) {
                            const float4 v = s4[rec_nb(r4, k)];
                            nx[k] = v.x;
                            ny[k] = v.y;
                            nz[k] = v.z;
                        }
                        const float4 v = s4[t];
                        float tx, ty, tz;
                        if (heis_attempt<ND, DK>(m, v.x, v.y, v.z, nx, ny, nz, sp[sl], r, tx, ty, tz))
                            s4[t] = make_float4(tx, ty, tz, 0.0f);
                    }
                }
                __syncthreads();
            }
        }
        if constexpr (MEASURE) {
            __shared__ float wred[kMaxSlots][kNP];
            const int nw = blockDim.x >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
            const int gw = max(1, nw / nslot), ngroups = nw / gw;   // warps per slot, groups
            const int grp = warp / gw, wig = warp - grp * gw;
            // wred row sl * gw + wig < max(nw, nslot) <= kMaxSlots
            for (int sl = grp; sl < nslot && grp < ngroups; sl += ngroups) {
                float acc[kNP];
#pragma unroll
                for (int k = 0; k < kNP; ++k) acc[k] = 0.0f;
                if (sch[sl] >= 0) {
                    const int rb = fm.slot_red[c0 + sl], re = (sl + 1 < nslot) ? fm.slot_red[c0 + sl + 1] : nred;
                    const int bb = fm.slot_black[c0 + sl], be = (sl + 1 < nslot) ? fm.slot_black[c0 + sl + 1] : n;
                    const int nr = re - rb, ns = nr + (be - bb);
#pragma unroll 1
                    for (int i = wig * 32 + lane; i < ns; i += gw * 32) {
                        const int t = (i < nr) ? rb + i : bb + (i - nr);
                        resident_site_terms<ISING>(m, t, i < nr, sx, s4, rec[t], cap, acc);
                    }
                }
#pragma unroll
                for (int k = 0; k < kNP; ++k) {
                    float v = acc[k];
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
                    if (lane == 0) wred[sl * gw + wig][k] = v;
                }
            }
            __syncthreads();
            // one warp per slot: lane k sums total k over the slot's warps in FP64, in warp order
            for (int sl = warp; sl < nslot; sl += nw) {
                const int ch = sch[sl];   // the same for the whole warp
                if (ch < 0) continue;
                double v = 0.0;
                if (lane < kNP)
                    for (int w = 0; w < gw; ++w) v += (double)wred[sl * gw + w][lane];
                const int ci = fm.pos ? fm.pos[ch] : ch;
                const double qv = ISING ? 0.0 : __shfl_sync(0xffffffffu, v, 10) / (2 * M_PI);
                if (fm.q && lane == 0) fm.q[ci] = qv;
                finalize_chain_warp(v, lane, fm.Hd + 3 * (size_t)ch, qv, fm.obs + (size_t)ci * NMMC_OBS_N,
                                    fm.acc + (size_t)ch * NMMC_ACC_N, fm.accumulate);
            }
        }
        for (int t = threadIdx.x; t < n; t += blockDim.x) {
            if (sch[rec[t].w >> kBoxBits] < 0) continue;
            const uint32_t off = a.goff[s0 + t];
            if (ISING) {
                ((int8_t*)a.spins)[off] = (int8_t)sx[t];
            } else {
                float* f = (float*)a.spins;
                const float4 v = s4[t];
                f[off] = v.x;
                f[off + P] = v.y;
                f[off + 2 * P] = v.z;
            }
        }
        for (int t = threadIdx.x; t < nslot; t += blockDim.x)
            if (sch[t] >= 0) a.sweep[sch[t]] += (unsigned long long)a.nsweeps;
        __syncthreads();
    }
}

// ------------------------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------------------------
namespace {

int site_bytes(const Ctx& c) { return c.ising ? 4 : 16; }

// Dynamic shared memory of a launch: the bin's spins (+ the zero site); the drawn-ahead
// variant adds its two buffers of Philox words.
size_t dyn_smem(const Ctx& c, bool pre) {
    if (!pre) return (size_t)(c.res.cap + 1) * site_bytes(c);
    return draw_smem_offset(c.res.cap, site_bytes(c)) + 2 * (size_t)c.res.cap * sizeof(uint4);
}

size_t smem_budget(const Ctx& c) {
    // per-slot parameters, counters and chain ids, the fused measurement's sums, the zero site
    size_t static_bytes = kMaxSlots * (sizeof(float4) + sizeof(unsigned long long) + sizeof(int)) +
                          kMaxSlots * kNP * sizeof(float) + 64 + 16;
    return c.smem_optin > static_bytes ? c.smem_optin - static_bytes : 0;
}

// LPT packing of chains into nb bins of at most cap sites and kMaxSlots chains.
bool pack_bins(const std::vector<int>& load, int nb, int cap, std::vector<std::vector<int>>& bins) {
    std::vector<int> order(load.size());
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return load[a] > load[b]; });
    bins.assign(nb, {});
    std::vector<long> bl(nb, 0);
    for (int ch : order) {
        int best = -1;
        for (int b = 0; b < nb; ++b) {
            if ((int)bins[b].size() >= kMaxSlots || bl[b] + load[ch] > cap) continue;
            if (best < 0 || bl[b] < bl[best]) best = b;
        }
        if (best < 0) return false;
        bins[best].push_back(ch);
        bl[best] += load[ch];
    }
    // drop empty bins
    bins.erase(std::remove_if(bins.begin(), bins.end(), [](const std::vector<int>& v) { return v.empty(); }),
               bins.end());
    return true;
}

void free_tables(ResidentTables& r) {
    cudaFree(r.d_site_chain);
    cudaFree(r.d_draws);
    r.d_site_chain = nullptr;
    r.d_draws = nullptr;
    r.draw_sweeps = 0;
    r.predraw = false;
    cudaFree(r.d_goff);
    cudaFree(r.d_rec);
    cudaFree(r.d_bin_begin);
    cudaFree(r.d_bin_nred);
    cudaFree(r.d_bin_chain_begin);
    cudaFree(r.d_bin_chains);
    cudaFree(r.d_slot_red);
    cudaFree(r.d_slot_black);
    r.d_goff = nullptr;
    r.d_rec = nullptr;
    r.d_bin_begin = r.d_bin_nred = r.d_bin_chain_begin = r.d_bin_chains = nullptr;
    r.d_slot_red = r.d_slot_black = nullptr;
    r.built = false;
    r.stencil = false;
    r.hbm_faster = false;
    r.tables_bins = 0;
}

template <class T>
int upload(T** dst, const std::vector<T>& v) {
    size_t bytes = std::max<size_t>(1, v.size()) * sizeof(T);
    cudaError_t e = cudaMalloc((void**)dst, bytes);
    if (e != cudaSuccess) return cuda_check(e, "cudaMalloc(resident table)");
    if (!v.empty()) {
        e = cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cuda_check(e, "cudaMemcpy(resident table)");
    }
    return NMMC_OK;
}

// Builds the site tables for a bin assignment (the CTA width is set separately).
int build_tables(Ctx& c, const std::vector<std::vector<int>>& bins) {
    ResidentTables& r = c.res;
    free_tables(r);
    const int E = c.edge, nz = (c.dim == 3) ? E : 1, ND = 2 * c.dim;
    const int ncomp = c.ising ? 1 : 3;
    const size_t P = (size_t)c.m.nhalf_pad;
    if ((uint64_t)c.box_sites > kBoxMask + 1ull)
        return set_error(NMMC_ERR_UNSUPPORTED, "box too large for the resident path");
    std::vector<uint32_t> goff;
    std::vector<uint4> rec;
    std::vector<int> site_chain;
    std::vector<int> bbeg{0}, bnred, bcbeg{0}, bch, sred, sblack;
    int cap = 0;
    for (const auto& bin : bins) {
        // local numbering: colour 0 sites of every chain, then colour 1
        std::vector<std::pair<int, int>> order;   // (chain slot, box)
        std::vector<int> first[2];                // per slot: first bin-local site of each colour
        int nred = 0;
        for (int colour = 0; colour < 2; ++colour)
            for (size_t s = 0; s < bin.size(); ++s) {
                int ch = bin[s];
                first[colour].push_back((int)order.size());
                const uint8_t* mk = c.masked ? &c.mask[(size_t)ch * c.box_sites] : nullptr;
                for (int z = 0; z < nz; ++z)
                    for (int y = 0; y < E; ++y)
                        for (int x = 0; x < E; ++x) {
                            if (((x + y + z) & 1) != colour) continue;
                            long box = x + (long)E * (y + (long)E * z);
                            if (mk && !mk[box]) continue;
                            order.push_back({(int)s, (int)box});
                            if (colour == 0) nred++;
                        }
            }
        const int n = (int)order.size();
        if (n > 65534) return set_error(NMMC_ERR_UNSUPPORTED, "resident bin too large");
        cap = std::max(cap, n);
        // index lookup per slot
        std::vector<std::vector<int>> lut(bin.size());
        for (size_t s = 0; s < bin.size(); ++s) lut[s].assign((size_t)c.box_sites, -1);
        for (int t = 0; t < n; ++t) lut[order[t].first][order[t].second] = t;
        for (int t = 0; t < n; ++t) {
            int s = order[t].first, box = order[t].second, ch = bin[s];
            int x = box % E, y = (box / E) % E, z = box / (E * E);
            int colour = (x + y + z) & 1;
            uint32_t i = (uint32_t)((z * c.m.ly + y) * c.m.hx + (x >> 1));
            size_t o = ((size_t)ch * 2 + colour) * ncomp * P + i;
            if (o > 0xFFFFFFFFull) return set_error(NMMC_ERR_UNSUPPORTED, "spin array too large for the resident path");
            goff.push_back((uint32_t)o);
            uint16_t j[6] = {kNoNb, kNoNb, kNoNb, kNoNb, kNoNb, kNoNb};
            for (int k = 0; k < ND; ++k) {
                int q[3] = {x + (k == 0) - (k == 1), y + (k == 2) - (k == 3), z + (k == 4) - (k == 5)};
                bool ok = true;
                for (int a = 0; a < c.dim; ++a) {
                    if (c.periodic) q[a] = (q[a] + E) % E;
                    else if (q[a] < 0 || q[a] >= E) ok = false;
                }
                int v = ok ? lut[s][q[0] + E * (q[1] + E * q[2])] : -1;
                if (v >= 0) j[k] = (uint16_t)v;
            }
            uint4 rr;
            rr.x = j[0] | ((uint32_t)j[1] << 16);
            rr.y = j[2] | ((uint32_t)j[3] << 16);
            rr.z = j[4] | ((uint32_t)j[5] << 16);
            rr.w = (uint32_t)box | ((uint32_t)s << kBoxBits);
            rec.push_back(rr);
            site_chain.push_back(ch);
        }
        bbeg.push_back(bbeg.back() + n);
        bnred.push_back(nred);
        for (int ch : bin) bch.push_back(ch);
        bcbeg.push_back((int)bch.size());
        sred.insert(sred.end(), first[0].begin(), first[0].end());
        sblack.insert(sblack.end(), first[1].begin(), first[1].end());
    }
    // absent neighbours -> the zero site (index cap, past every bin's last site)
    for (uint4& rr : rec)
        for (uint32_t* w : {&rr.x, &rr.y, &rr.z}) {
            uint32_t lo = *w & 0xFFFFu, hi = *w >> 16;
            if (lo == kNoNb) lo = (uint32_t)cap;
            if (hi == kNoNb) hi = (uint32_t)cap;
            *w = lo | (hi << 16);
        }
    int rc;
    if ((rc = upload(&r.d_goff, goff)) || (rc = upload(&r.d_rec, rec)) || (rc = upload(&r.d_bin_begin, bbeg)) ||
        (rc = upload(&r.d_bin_nred, bnred)) || (rc = upload(&r.d_bin_chain_begin, bcbeg)) ||
        (rc = upload(&r.d_bin_chains, bch)) || (rc = upload(&r.d_slot_red, sred)) ||
        (rc = upload(&r.d_slot_black, sblack)) || (rc = upload(&r.d_site_chain, site_chain)))
        return rc;
    r.nbins = (int)bins.size();
    r.cap = cap;
    r.total_sites = bbeg.back();
    r.tables_bins = (int)bins.size();
    return NMMC_OK;
}

// The instantiation a context launches (fused: the 2-D sweep + observables variant; pre: the
// drawn-ahead variant, 2-D only).
template <int DIM, bool ISING, bool MEASURE, bool PRE>
const void* kernel_dk(int dk) {
    if (ISING) return (const void*)k_resident<DIM, kDmiNone, true, MEASURE, PRE>;
    switch (dk) {
        case kDmiNone: return (const void*)k_resident<DIM, kDmiNone, false, MEASURE, PRE>;
        case kDmiGeneral: return (const void*)k_resident<DIM, kDmiGeneral, false, MEASURE, PRE>;
        case kDmiPairs: return (const void*)k_resident<DIM, kDmiPairs, false, MEASURE, PRE>;
        default: return (const void*)k_resident<DIM, kDmiAxial, false, MEASURE, PRE>;
    }
}

const void* kernel_for(const Ctx& c, bool fused, bool pre) {
    const int dk = c.m.dmi_kind;
    if (c.dim == 3) return c.ising ? kernel_dk<3, true, false, false>(dk) : kernel_dk<3, false, false, false>(dk);
    if (pre) {
        if (fused) return c.ising ? kernel_dk<2, true, true, true>(dk) : kernel_dk<2, false, true, true>(dk);
        return c.ising ? kernel_dk<2, true, false, true>(dk) : kernel_dk<2, false, false, true>(dk);
    }
    if (fused) return c.ising ? kernel_dk<2, true, true, false>(dk) : kernel_dk<2, false, true, false>(dk);
    return c.ising ? kernel_dk<2, true, false, false>(dk) : kernel_dk<2, false, false, false>(dk);
}

// Sites per sweep row of the drawn-ahead buffer at most (16 B each), and its size.
constexpr long long kPredrawMaxSites = 1 << 19;
constexpr size_t kPredrawBytes = 32u << 20;

// The drawn-ahead variant applies: 2-D tables, its buffers fit in shared memory, and one sweep
// of words for every site is at most kPredrawMaxSites rows.
bool predraw_fits(const Ctx& c) {
    return c.dim == 2 && c.res.total_sites > 0 && c.res.total_sites <= kPredrawMaxSites &&
           dyn_smem(c, true) <= smem_budget(c);
}

int set_attr(Ctx& c) {
    for (bool pre : {false, true}) {
        if (pre && !predraw_fits(c)) continue;
        for (bool fused : {false, true}) {
            if (fused && c.dim == 3) continue;
            int rc = cuda_check(cudaFuncSetAttribute(kernel_for(c, fused, pre), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     (int)dyn_smem(c, pre)),
                                "cudaFuncSetAttribute(k_resident)");
            if (rc) return rc;
        }
    }
    return NMMC_OK;
}

// The drawn-ahead buffer: as many sweeps of words as kPredrawBytes holds (at least one, at
// most 256); calls with more sweeps are split.
int ensure_draws(Ctx& c) {
    ResidentTables& r = c.res;
    if (r.d_draws) return NMMC_OK;
    const size_t row = (size_t)r.total_sites * sizeof(uint4);
    r.draw_sweeps = (int)std::max<size_t>(1, std::min<size_t>(256, kPredrawBytes / row));
    cudaError_t e = cudaMalloc((void**)&r.d_draws, row * r.draw_sweeps);
    if (e != cudaSuccess) {
        r.d_draws = nullptr;
        r.draw_sweeps = 0;
        return cuda_check(e, "cudaMalloc(drawn-ahead words)");
    }
    return NMMC_OK;
}

// Persistent grid: as many CTAs as fit on the GPU at once (by the occupancy of the kernel
// that is launched), at most one per bin; CTAs loop over the remaining bins. 0: cannot launch.
int grid_for(const Ctx& c, bool fused, bool pre) {
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel_for(c, fused, pre), c.res.threads,
                                                      dyn_smem(c, pre)) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    if (occ < 1) return 0;
    return std::min(c.res.nbins, occ * c.sm_count);
}

ResidentArgs make_args(Ctx& c, int nsweeps) {
    const ResidentTables& r = c.res;
    return ResidentArgs{c.d_spins, c.d_bh, c.d_sweep, c.d_active, r.d_goff, r.d_rec, r.d_bin_begin, r.d_bin_nred,
                        r.d_bin_chain_begin, r.d_bin_chains, r.nbins, r.cap, nsweeps, r.d_draws,
                        (long long)r.total_sites};
}

int launch_one(Ctx& c, int nsweeps, const FusedMeasure* fm, bool pre) {
    const bool fused = fm != nullptr;
    const int grid = grid_for(c, fused, pre);
    if (grid <= 0) return set_error(NMMC_ERR_UNSUPPORTED, "resident kernel does not fit on an SM");
    ResidentArgs a = make_args(c, nsweeps);
    FusedMeasure none{};
    DevModel m = c.m;
    void* args[] = {&m, &a, fused ? (void*)const_cast<FusedMeasure*>(fm) : (void*)&none};
    return cuda_check(cudaLaunchKernel(kernel_for(c, fused, pre), dim3(grid), dim3(c.res.threads), args,
                                       dyn_smem(c, pre), c.stream),
                      "k_resident launch");
}

// Kernel launches of do_launch for nsweeps sweeps (the drawn-ahead variant launches k_predraw
// before each resident launch and splits long calls).
int launches_for(const Ctx& c, int nsweeps) {
    if (!c.res.predraw || nsweeps <= 0) return 1;
    return 2 * ((nsweeps + c.res.draw_sweeps - 1) / c.res.draw_sweeps);
}

int do_launch(Ctx& c, int nsweeps, const FusedMeasure* fm) {
    ResidentTables& r = c.res;
    if (!r.predraw || nsweeps <= 0) return launch_one(c, nsweeps, fm, false);
    if (!r.d_draws || r.draw_sweeps < 1) return set_error(NMMC_ERR_UNSUPPORTED, "drawn-ahead buffer missing");
    for (int done = 0; done < nsweeps;) {
        const int k = std::min(nsweeps - done, r.draw_sweeps);
        const long long items = (long long)r.total_sites * k;
        const int blocks = (int)std::min<long long>((items + 255) / 256, 8LL * c.sm_count);
        k_predraw<<<blocks, 256, 0, c.stream>>>(c.m, r.d_rec, r.d_site_chain, c.d_active, c.d_sweep, r.d_draws,
                                                r.total_sites, k);
        int rc = cuda_check(cudaGetLastError(), "k_predraw launch");
        if (rc) return rc;
        done += k;
        if ((rc = launch_one(c, k, done == nsweeps ? fm : nullptr, true))) return rc;
    }
    return NMMC_OK;
}

std::string cache_path() {
    const char* d = getenv("NMMC_CACHE_DIR");
    std::string dir;
    if (d && *d) dir = d;
    else {
        const char* h = getenv("HOME");
        dir = std::string(h ? h : "/tmp") + "/.cache/nmmc_gb300";
    }
    std::string cmd = dir;
    // create the directory (one level below an existing parent is enough here)
    size_t pos = 0;
    while ((pos = cmd.find('/', pos + 1)) != std::string::npos) mkdir(cmd.substr(0, pos).c_str(), 0755);
    mkdir(dir.c_str(), 0755);
    return dir + "/resident_autotune.txt";
}

std::string config_key(const Ctx& c) {
    // hash of the model and of the per-chain site counts, plus the GPU name
    uint64_t h = 1469598103934665603ull;
    auto mix = [&](uint64_t v) {
        h ^= v;
        h *= 1099511628211ull;
    };
    mix((uint64_t)c.dim);
    mix((uint64_t)c.edge);
    mix((uint64_t)c.ising);
    mix((uint64_t)c.periodic);
    mix((uint64_t)c.masked);
    mix((uint64_t)c.m.has_dmi);
    for (int v : c.num) mix((uint64_t)v);
    mix((uint64_t)c.m.dmi_kind);
    mix(6);   // table and kernel format (5: the path choice, stencil kernel included, is part of the entry;
              // 6: 16 bytes of shared memory per Heisenberg site)
    std::string g = c.gpu_name;
    for (char& ch : g)
        if (ch == ' ') ch = '_';
    char buf[64];
    snprintf(buf, sizeof buf, "%016llx", (unsigned long long)h);
    return g + ":" + buf;
}

// Cache lines: key, bins, threads, drawn-ahead (0/1), path (0 the record kernel, 1 the HBM
// path, 2 the stencil kernel); the last line of a key wins. Lines of another format are skipped.
bool cache_lookup(const std::string& key, int& nbins, int& threads, int& pre, int& hbm) {
    std::ifstream f(cache_path());
    std::string line;
    bool found = false;
    while (std::getline(f, line)) {
        std::istringstream ls(line);
        std::string k, extra;
        int b, t, p, h;
        if (!(ls >> k >> b >> t >> p >> h) || (ls >> extra) || k != key) continue;
        nbins = b;
        threads = t;
        pre = p;
        hbm = h;
        found = true;
    }
    return found;
}

void cache_store(const std::string& key, int nbins, int threads, int pre, int hbm) {
    std::ofstream f(cache_path(), std::ios::app);
    if (f) f << key << " " << nbins << " " << threads << " " << pre << " " << hbm << "\n";
}

}  // namespace

void resident_free(Ctx& c) { free_tables(c.res); }

int resident_launches(const Ctx& c, int nsweeps) { return c.res.stencil ? 1 : launches_for(c, nsweeps); }

// Decides eligibility and builds the tables (autotuned unless options fix the shape).
int resident_prepare(Ctx& c) {
    if (c.res.built) return NMMC_OK;
    const size_t budget = smem_budget(c);
    const int cap_sites = (int)std::min<size_t>(65534, budget / site_bytes(c) - 1);
    int maxn = 0;
    for (int v : c.num) maxn = std::max(maxn, v);
    // general interaction tables use the multi-colour gather sweep
    c.res.eligible = maxn > 0 && maxn <= cap_sites && !c.m.general;
    if (!c.res.eligible) return NMMC_OK;
    // the stencil kernel covers unmasked 2-D Heisenberg lattices that fit one chain per CTA
    const bool stencil_ok = c.res_stencil != 1 && stencil_slots(c, c.nchains) > 0;

    std::vector<int> load(c.num.begin(), c.num.end());
    auto tables_for = [&](int nbins) -> int {
        if (c.res.tables_bins == nbins && c.res.d_rec) return NMMC_OK;
        std::vector<std::vector<int>> bins;
        if (!pack_bins(load, nbins, cap_sites, bins)) return NMMC_ERR_UNSUPPORTED;
        int rc = build_tables(c, bins);
        if (rc) return rc;
        c.res.tables_bins = nbins;
        return set_attr(c);
    };
    // drawn-ahead variant for a bin count: off by option or where it does not fit; on by option
    // where it fits; otherwise both are candidates (autotuned) when the bins leave SMs idle
    auto pre_choices = [&](int nbins) -> std::vector<bool> {
        if (c.res_predraw == 1 || !predraw_fits(c)) return {false};
        if (c.res_predraw == 2) return {true};
        if (nbins > c.sm_count) return {false};
        return {false, true};
    };
    auto finish = [&](int nbins, int threads, bool pre) -> int {
        int rc = tables_for(nbins);
        if (rc) return rc;
        c.res.threads = threads;
        c.res.predraw = pre && predraw_fits(c);
        if (c.res.predraw && (rc = ensure_draws(c))) return rc;
        if (grid_for(c, false, c.res.predraw) <= 0 || (c.dim == 2 && grid_for(c, true, c.res.predraw) <= 0) ||
            grid_for(c, false, false) <= 0 || (c.dim == 2 && grid_for(c, true, false) <= 0))
            return set_error(NMMC_ERR_UNSUPPORTED, "resident kernel of %d threads does not fit on an SM", threads);
        c.res.built = true;
        return NMMC_OK;
    };

    int fixed_bins = c.res_bins, fixed_threads = c.res_threads;
    if (fixed_bins > 0 && fixed_threads > 0) {
        // no timing: the drawn-ahead variant where the option asks for it, or (automatic) where
        // the bins occupy at most half of the SMs
        const int nb = std::min(fixed_bins, c.nchains);
        int rc = tables_for(nb);
        if (rc) return rc;
        const std::vector<bool> pc = pre_choices(nb);
        const bool pre = pc.size() == 1 ? pc[0] : 2 * nb <= c.sm_count;
        rc = finish(nb, fixed_threads, pre);
        c.res.stencil = rc == NMMC_OK && c.res_stencil == 2 && stencil_ok;
        return rc;
    }

    // candidate shapes
    long total = std::accumulate(load.begin(), load.end(), 0L);
    int min_bins = (int)std::max<long>(1, (total + cap_sites - 1) / cap_sites);
    std::vector<int> cand_bins;
    for (int k : {1, 2, 3, 4}) cand_bins.push_back(std::min(c.nchains, std::max(min_bins, k * c.sm_count)));
    cand_bins.push_back(c.nchains);
    std::sort(cand_bins.begin(), cand_bins.end());
    cand_bins.erase(std::unique(cand_bins.begin(), cand_bins.end()), cand_bins.end());
    std::vector<int> cand_threads;
    for (int t = 128; t <= 1024; t += 64) cand_threads.push_back(t);
    if (fixed_bins > 0) cand_bins = {std::min(fixed_bins, c.nchains)};
    if (fixed_threads > 0) cand_threads = {fixed_threads};

    // a cached shape is used when it agrees with the options that fix part of it; only fully
    // automatic choices are stored
    const bool automatic = fixed_bins <= 0 && fixed_threads <= 0 && c.res_predraw == 0 && c.res_stencil == 0;
    const std::string key = config_key(c);
    int cb = 0, ct = 0, cp = 0, ch = 0;
    if (cache_lookup(key, cb, ct, cp, ch) &&
        (fixed_bins <= 0 || cb == std::min(fixed_bins, c.nchains)) && (fixed_threads <= 0 || ct == fixed_threads) &&
        (c.res_predraw == 0 || (c.res_predraw == 2) == (cp != 0)) && finish(cb, ct, cp != 0) == NMMC_OK) {
        c.res.hbm_faster = automatic && ch == 1;
        c.res.stencil = (automatic && ch == 2 && c.res_stencil == 0) || (c.res_stencil == 2 && stencil_ok);
        return NMMC_OK;
    }

    // time each candidate on the live chains, with the variant the sampling loop launches
    // (2-D: sweeps + observables); spins and counters are restored afterwards
    const bool fused = c.dim == 2 && !c.measure_fp64;
    DeviceScratch ds;
    void* snap = nullptr;
    unsigned long long* snap_sw = nullptr;
    NMMC_CUDA(ds.alloc(&snap, c.spins_bytes));
    NMMC_CUDA(ds.alloc(&snap_sw, sizeof(unsigned long long) * c.nchains));
    NMMC_CUDA(cudaMemcpyAsync(snap, c.d_spins, c.spins_bytes, cudaMemcpyDeviceToDevice, c.stream));
    NMMC_CUDA(cudaMemcpyAsync(snap_sw, c.d_sweep, sizeof(unsigned long long) * c.nchains,
                              cudaMemcpyDeviceToDevice, c.stream));
    NMMC_CUDA(cudaMemsetAsync(c.d_active, 1, c.nchains, c.stream));
    int rc = upload_params(c);
    if (rc) return rc;
    cudaEvent_t ea, eb;
    cudaEventCreate(&ea);
    cudaEventCreate(&eb);
    float best = 1e30f;
    int best_b = 0, best_t = 0;
    bool best_p = false;
    for (int nb : cand_bins) {
        if (tables_for(nb) != NMMC_OK) continue;
        FusedMeasure fm{c.d_obs, c.d_q, c.d_acc, c.d_Hd, nullptr, c.res.d_slot_red, c.res.d_slot_black, 0};
        for (bool pre : pre_choices(nb))
        for (int th : cand_threads) {
            c.res.threads = th;
            c.res.predraw = pre;
            if (pre && ensure_draws(c) != NMMC_OK) continue;
            if (grid_for(c, fused, pre) <= 0) continue;
            if (do_launch(c, 1, fused ? &fm : nullptr) != NMMC_OK) continue;   // warm-up
            float ms = 1e30f;
            bool ok = true;
            for (int rep = 0; rep < 3 && ok; ++rep) {   // best of three short runs
                cudaEventRecord(ea, c.stream);
                do_launch(c, 8, fused ? &fm : nullptr);
                cudaEventRecord(eb, c.stream);
                float t = 0;
                ok = cudaEventSynchronize(eb) == cudaSuccess && cudaEventElapsedTime(&t, ea, eb) == cudaSuccess &&
                     cudaGetLastError() == cudaSuccess;
                ms = std::min(ms, t);
            }
            if (!ok) continue;
            if (ms < best) {
                best = ms;
                best_b = nb;
                best_t = th;
                best_p = pre;
            }
        }
    }
    c.res.predraw = false;
    // the HBM path as one more candidate of the automatic choice: the same sweeps and
    // observables on the streaming kernels (at few large lattices a resident kernel occupies
    // few SMs: 16 chains of 128^2 sweep in 8.6 us there against 16.6 us resident)
    bool hbm = false;
    if (automatic && c.sweep_path == 0 && best_b > 0 && hbm_tuning_step(c, 1, fused) == NMMC_OK) {
        float ms = 1e30f;
        bool ok = true;
        for (int rep = 0; rep < 3 && ok; ++rep) {
            cudaEventRecord(ea, c.stream);
            ok = hbm_tuning_step(c, 8, fused) == NMMC_OK;
            cudaEventRecord(eb, c.stream);
            float t = 0;
            ok = ok && cudaEventSynchronize(eb) == cudaSuccess && cudaEventElapsedTime(&t, ea, eb) == cudaSuccess &&
                 cudaGetLastError() == cudaSuccess;
            ms = std::min(ms, t);
        }
        hbm = ok && ms < best;
        if (hbm) best = ms;
    }
    // the stencil kernel: timed on the automatic choice, taken without timing when forced
    bool stencil = c.res_stencil == 2 && stencil_ok;
    if (c.res_stencil == 0 && stencil_ok && best_b > 0 &&
        launch_stencil_sweeps(c, c.d_all, c.nchains, 1, fused, 0) == NMMC_OK) {
        float ms = 1e30f;
        bool ok = true;
        for (int rep = 0; rep < 3 && ok; ++rep) {
            cudaEventRecord(ea, c.stream);
            ok = launch_stencil_sweeps(c, c.d_all, c.nchains, 8, fused, 0) == NMMC_OK;
            cudaEventRecord(eb, c.stream);
            float t = 0;
            ok = ok && cudaEventSynchronize(eb) == cudaSuccess && cudaEventElapsedTime(&t, ea, eb) == cudaSuccess &&
                 cudaGetLastError() == cudaSuccess;
            ms = std::min(ms, t);
        }
        if (ok && ms < best) {
            stencil = true;
            hbm = false;
        }
    }
    cudaGetLastError();
    cudaEventDestroy(ea);
    cudaEventDestroy(eb);
    NMMC_CUDA(cudaMemcpyAsync(c.d_spins, snap, c.spins_bytes, cudaMemcpyDeviceToDevice, c.stream));
    NMMC_CUDA(cudaMemcpyAsync(c.d_sweep, snap_sw, sizeof(unsigned long long) * c.nchains, cudaMemcpyDeviceToDevice,
                              c.stream));
    NMMC_CUDA(cudaStreamSynchronize(c.stream));
    c.active_all = true;   // every chain marked active above
    if (best_b == 0) {
        c.res.eligible = false;
        return NMMC_OK;
    }
    if (automatic) cache_store(key, best_b, best_t, best_p ? 1 : 0, stencil ? 2 : (hbm ? 1 : 0));
    rc = finish(best_b, best_t, best_p);
    c.res.hbm_faster = hbm;
    c.res.stencil = stencil;
    return rc;
}

bool resident_chosen(const Ctx& c) {
    return c.res.eligible && !(c.sweep_path == 0 && c.res.hbm_faster);
}

__global__ void k_mark_active(uint8_t* active, int* pos, const int* chains, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        active[chains[i]] = 1;
        pos[chains[i]] = i;
    }
}

bool resident_can_measure(const Ctx& c) {
    // one z-slice, FP32 observables, and whole warps for the per-slot reductions
    return c.res.built && c.res.eligible && c.dim == 2 && !c.measure_fp64 && c.res.threads >= 32 &&
           c.res.threads % 32 == 0;
}

int launch_resident_sweeps(Ctx& c, const int* d_chains, int n, int nsweeps, bool all, bool measure,
                           int accumulate) {
    if (c.res.stencil) {   // whole chains from the list: no chain marks needed
        if (measure && !resident_can_measure(c)) return set_error(NMMC_ERR_UNSUPPORTED, "fused measurement not available");
        return launch_stencil_sweeps(c, d_chains, n, nsweeps, measure, accumulate);
    }
    // Mark the chains of this call; the others keep their spins and counters. A direct call on
    // every chain reuses the marks of the previous such call; a captured launch always writes
    // them, since a graph may be replayed after other calls have changed them.
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    NMMC_CUDA(cudaStreamIsCapturing(c.stream, &cs));
    const bool direct_all = all && cs == cudaStreamCaptureStatusNone;
    if (direct_all) {
        if (!c.active_all) NMMC_CUDA(cudaMemsetAsync(c.d_active, 1, c.nchains, c.stream));
        c.active_all = true;
    } else {
        NMMC_CUDA(cudaMemsetAsync(c.d_active, 0, c.nchains, c.stream));
        k_mark_active<<<(n + 127) / 128, 128, 0, c.stream>>>(c.d_active, c.d_pos, d_chains, n);
        c.active_all = false;
    }
    if (!measure) return do_launch(c, nsweeps, nullptr);
    if (!resident_can_measure(c)) return set_error(NMMC_ERR_UNSUPPORTED, "fused measurement not available");
    FusedMeasure fm{c.d_obs, c.d_q, c.d_acc, c.d_Hd, direct_all ? nullptr : c.d_pos,
                    c.res.d_slot_red, c.res.d_slot_black, accumulate};
    return do_launch(c, nsweeps, &fm);
}

}  // namespace nmmc
