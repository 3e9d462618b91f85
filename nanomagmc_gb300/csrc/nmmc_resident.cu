// Shared-memory resident checkerboard sweeps for lattices that fit on chip: the 2-D runs and
// the batched Weibull nanoparticles. One persistent CTA owns a "bin" of whole chains: it
// loads their filled sites into shared memory once, runs all requested sweeps there with a
// __syncthreads between colours, and writes the spins back once. This replaces the
// reference's MPI split over lattices, temperatures and fields (Old/lib/main.cpp:104-275,
// Old/lib/protocol.cpp:97-131): every chain of the batch is a slot in some bin.
//
// Sites are stored compactly (only filled sites, colour 0 first), with a per-site table of
// bin-local neighbour indices, so uneven particle sizes cost only their own sites. Bins are
// packed longest-processing-time first; the bin count and CTA width are chosen by timing
// candidates on the live context (autotune) and cached per (model, sizes, GPU).
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

constexpr int kMaxSlots = 64;
constexpr uint16_t kNoNb = 0xFFFF;

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
template <bool ISING>
__device__ __forceinline__ void resident_site_terms(const DevModel& m, int t, int g, bool red,
                                                    const float* sx, const float* sy, const float* sz,
                                                    const uint32_t* __restrict__ sbox,
                                                    const uint16_t* __restrict__ nbr, int total_sites,
                                                    float* acc) {
    const float s0 = sx[t], s1 = ISING ? 0.0f : sy[t], s2 = ISING ? 0.0f : sz[t];
    // neighbours one at a time (few live registers); the triangles re-read theirs below
    float f0 = 0.f, f1 = 0.f, f2 = 0.f;
    uint16_t j[4];
#pragma unroll
    for (int d = 0; d < 4; ++d) {
        j[d] = nbr[(size_t)d * total_sites + g];
        if (j[d] == kNoNb) continue;
        const float J = m.J[d];
        const float n0 = sx[j[d]];
        f0 = fmaf(J, n0, f0);
        if (!ISING) {
            const float n1 = sy[j[d]], n2 = sz[j[d]];
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
    const int box = (int)sbox[g];
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
        const bool pq = m.periodic && m.periodic_q;
        const bool qxp = j[0] != kNoNb && (x + 1 < m.edge || pq), qxm = j[1] != kNoNb && (x >= 1 || pq);
        const bool qyp = j[2] != kNoNb && (y + 1 < m.edge || pq), qym = j[3] != kNoNb && (y >= 1 || pq);
        if (qxm && qyp)
            acc[10] += solid_angle_f(s0, s1, s2, sx[j[1]], sy[j[1]], sz[j[1]], sx[j[2]], sy[j[2]], sz[j[2]]);
        if (qxp && qym)
            acc[10] += solid_angle_f(s0, s1, s2, sx[j[0]], sy[j[0]], sz[j[0]], sx[j[3]], sy[j[3]], sz[j[3]]);
    }
}

// Register bound of the fused (MEASURE) variants, as blocks of 1024 threads per SM: 0 leaves
// the choice to the compiler (about 56 registers: one 1024-thread or two 512-thread blocks
// per SM); 2 holds them to 32 registers with some spilling. Measured on GB300, 0 is 1-4%
// faster on the batched-grain and 2-D workloads.
#ifndef NMMC_FUSED_MIN_BLOCKS
#define NMMC_FUSED_MIN_BLOCKS 0
#endif

// MEASURE: after the last sweep, the bin's observables are computed from the spins still in
// shared memory and written straight to the outputs (no partial-sum pass over HBM). Each
// chain slot is summed by a fixed group of warps: FP32 per thread and per warp, FP64 across
// the group's warps in a fixed order, so results are reproducible run to run.
template <int DIM, int DK, bool ISING, bool MEASURE>
__global__ void __launch_bounds__(1024, MEASURE ? NMMC_FUSED_MIN_BLOCKS : 0)
k_resident(const DevModel m, void* __restrict__ spins_v, const float4* __restrict__ bh,
           unsigned long long* __restrict__ sweep, const uint8_t* __restrict__ active,
           const uint32_t* __restrict__ goff, const uint32_t* __restrict__ sbox,
           const uint16_t* __restrict__ slot, const uint16_t* __restrict__ nbr, int total_sites,
           const int* __restrict__ bin_begin, const int* __restrict__ bin_nred,
           const int* __restrict__ bin_cbeg, const int* __restrict__ bin_chains, int nbins, int cap,
           int nsweeps, const FusedMeasure fm) {
    static_assert(!MEASURE || DIM == 2, "the fused measurement covers one z-slice");
    extern __shared__ float sm[];
    __shared__ float4 sp[kMaxSlots];
    __shared__ unsigned long long ssw[kMaxSlots];
    __shared__ int sch[kMaxSlots];
    __shared__ uint8_t sact[kMaxSlots];
    constexpr int ND = 2 * DIM;
    const size_t P = (size_t)m.nhalf_pad;
    float* sx = sm;
    float* sy = sm + cap;
    float* sz = sm + 2 * cap;
    for (int b = blockIdx.x; b < nbins; b += gridDim.x) {
        const int s0 = bin_begin[b], n = bin_begin[b + 1] - s0, nred = bin_nred[b];
        const int c0 = bin_cbeg[b], nslot = bin_cbeg[b + 1] - c0;
        for (int t = threadIdx.x; t < nslot; t += blockDim.x) {
            int ch = bin_chains[c0 + t];
            sch[t] = ch;
            sp[t] = bh[ch];
            ssw[t] = sweep[ch];
            sact[t] = active[ch];
        }
        for (int t = threadIdx.x; t < n; t += blockDim.x) {
            uint32_t off = goff[s0 + t];
            if (ISING) {
                sx[t] = (float)((const int8_t*)spins_v)[off];
            } else {
                const float* f = (const float*)spins_v;
                sx[t] = f[off];
                sy[t] = f[off + P];
                sz[t] = f[off + 2 * P];
            }
        }
        __syncthreads();
        for (int sw = 0; sw < nsweeps; ++sw) {
            for (int colour = 0; colour < 2; ++colour) {
                const int lo = colour ? nred : 0, hi = colour ? n : nred;
                for (int t = lo + threadIdx.x; t < hi; t += blockDim.x) {
                    const int g = s0 + t;
                    const int sl = slot[g];
                    if (!sact[sl]) continue;
                    const nmmc_u4 r = sweep_draw(m, sbox[g], ssw[sl] + (unsigned)sw, (uint32_t)sch[sl]);
                    if (ISING) {
                        float nb[ND];
#pragma unroll
                        for (int k = 0; k < ND; ++k) {
                            uint16_t j = nbr[(size_t)k * total_sites + g];
                            nb[k] = (j != kNoNb) ? sx[j] : 0.0f;
                        }
                        float tnew;
                        if (ising_attempt<ND>(m, sx[t], nb, sp[sl], r, tnew)) sx[t] = tnew;
                    } else {
                        float nx[ND], ny[ND], nz[ND];
#pragma unroll
                        for (int k = 0; k < ND; ++k) {
                            uint16_t j = nbr[(size_t)k * total_sites + g];
                            if (j != kNoNb) {
                                nx[k] = sx[j];
                                ny[k] = sy[j];
                                nz[k] = sz[j];
                            } else {
                                nx[k] = ny[k] = nz[k] = 0.0f;
                            }
                        }
                        float tx, ty, tz;
                        if (heis_attempt<ND, DK>(m, sx[t], sy[t], sz[t], nx, ny, nz, sp[sl], r, tx, ty, tz)) {
                            sx[t] = tx;
                            sy[t] = ty;
                            sz[t] = tz;
                        }
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
                if (sact[sl]) {
                    const int rb = fm.slot_red[c0 + sl], re = (sl + 1 < nslot) ? fm.slot_red[c0 + sl + 1] : nred;
                    const int bb = fm.slot_black[c0 + sl], be = (sl + 1 < nslot) ? fm.slot_black[c0 + sl + 1] : n;
                    const int nr = re - rb, ns = nr + (be - bb);
#pragma unroll 1
                    for (int i = wig * 32 + lane; i < ns; i += gw * 32) {
                        const int t = (i < nr) ? rb + i : bb + (i - nr);
                        resident_site_terms<ISING>(m, t, s0 + t, i < nr, sx, sy, sz, sbox, nbr, total_sites, acc);
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
            for (int sl = threadIdx.x; sl < nslot; sl += blockDim.x) {
                if (!sact[sl]) continue;
                double tot[kNP];
#pragma unroll
                for (int k = 0; k < kNP; ++k) {
                    double v = 0;
                    for (int w = 0; w < gw; ++w) v += (double)wred[sl * gw + w][k];
                    tot[k] = v;
                }
                const int ch = sch[sl];
                const int ci = fm.pos ? fm.pos[ch] : ch;
                const double qv = ISING ? 0.0 : tot[10] / (2 * M_PI);
                if (fm.q) fm.q[ci] = qv;
                finalize_chain(tot, fm.Hd + 3 * (size_t)ch, qv, fm.obs + (size_t)ci * NMMC_OBS_N,
                               fm.acc + (size_t)ch * NMMC_ACC_N, fm.accumulate);
            }
        }
        for (int t = threadIdx.x; t < n; t += blockDim.x) {
            const int g = s0 + t;
            if (!sact[slot[g]]) continue;
            uint32_t off = goff[g];
            if (ISING) {
                ((int8_t*)spins_v)[off] = (int8_t)sx[t];
            } else {
                float* f = (float*)spins_v;
                f[off] = sx[t];
                f[off + P] = sy[t];
                f[off + 2 * P] = sz[t];
            }
        }
        for (int t = threadIdx.x; t < nslot; t += blockDim.x)
            if (sact[t]) sweep[sch[t]] += (unsigned long long)nsweeps;
        __syncthreads();
    }
}

// ------------------------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------------------------
namespace {

int site_bytes(const Ctx& c) { return c.ising ? 4 : 12; }

size_t smem_budget(const Ctx& c) {
    // per-slot parameters, counters, chain ids and flags, plus the fused measurement's sums
    size_t static_bytes = kMaxSlots * (sizeof(float4) + sizeof(unsigned long long) + sizeof(int) + 1) +
                          kMaxSlots * kNP * sizeof(float) + 64;
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
    cudaFree(r.d_goff);
    cudaFree(r.d_box);
    cudaFree(r.d_slot);
    cudaFree(r.d_nbr);
    cudaFree(r.d_bin_begin);
    cudaFree(r.d_bin_nred);
    cudaFree(r.d_bin_chain_begin);
    cudaFree(r.d_bin_chains);
    cudaFree(r.d_slot_red);
    cudaFree(r.d_slot_black);
    r.d_slot_red = r.d_slot_black = nullptr;
    r.d_goff = nullptr;
    r.d_box = nullptr;
    r.d_slot = nullptr;
    r.d_nbr = nullptr;
    r.d_bin_begin = r.d_bin_nred = r.d_bin_chain_begin = r.d_bin_chains = nullptr;
    r.built = false;
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

// Builds the site tables for a bin assignment.
int build_tables(Ctx& c, const std::vector<std::vector<int>>& bins, int threads) {
    ResidentTables& r = c.res;
    free_tables(r);
    const int E = c.edge, nz = (c.dim == 3) ? E : 1, ND = 2 * c.dim;
    const int ncomp = c.ising ? 1 : 3;
    const size_t P = (size_t)c.m.nhalf_pad;
    std::vector<uint32_t> goff, sbox;
    std::vector<uint16_t> slot;
    std::vector<std::vector<uint16_t>> nb(ND);
    std::vector<int> bbeg{0}, bnred, bcbeg{0}, bch, sred, sblack;
    std::vector<int> local((size_t)c.box_sites, -1);
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
            sbox.push_back((uint32_t)box);
            slot.push_back((uint16_t)s);
            for (int k = 0; k < ND; ++k) {
                int q[3] = {x + (k == 0) - (k == 1), y + (k == 2) - (k == 3), z + (k == 4) - (k == 5)};
                bool ok = true;
                for (int a = 0; a < c.dim; ++a) {
                    if (c.periodic) q[a] = (q[a] + E) % E;
                    else if (q[a] < 0 || q[a] >= E) ok = false;
                }
                int j = ok ? lut[s][q[0] + E * (q[1] + E * q[2])] : -1;
                nb[k].push_back(j >= 0 ? (uint16_t)j : kNoNb);
            }
        }
        bbeg.push_back(bbeg.back() + n);
        bnred.push_back(nred);
        for (int ch : bin) bch.push_back(ch);
        bcbeg.push_back((int)bch.size());
        sred.insert(sred.end(), first[0].begin(), first[0].end());
        sblack.insert(sblack.end(), first[1].begin(), first[1].end());
    }
    const int total = bbeg.back();
    std::vector<uint16_t> nbr((size_t)ND * total);
    for (int k = 0; k < ND; ++k) std::copy(nb[k].begin(), nb[k].end(), nbr.begin() + (size_t)k * total);
    int rc;
    if ((rc = upload(&r.d_goff, goff)) || (rc = upload(&r.d_box, sbox)) || (rc = upload(&r.d_slot, slot)) ||
        (rc = upload(&r.d_nbr, nbr)) || (rc = upload(&r.d_bin_begin, bbeg)) || (rc = upload(&r.d_bin_nred, bnred)) ||
        (rc = upload(&r.d_bin_chain_begin, bcbeg)) || (rc = upload(&r.d_bin_chains, bch)) ||
        (rc = upload(&r.d_slot_red, sred)) || (rc = upload(&r.d_slot_black, sblack)))
        return rc;
    r.nbins = (int)bins.size();
    r.cap = cap;
    r.threads = threads;
    r.total_sites = total;
    r.built = true;
    return NMMC_OK;
}

template <int DIM, int DK, bool ISING, bool MEASURE>
void res_launch(Ctx& c, int grid, int nsweeps, const FusedMeasure& fm) {
    ResidentTables& r = c.res;
    size_t smem = (size_t)r.cap * site_bytes(c);
    k_resident<DIM, DK, ISING, MEASURE><<<grid, r.threads, smem, c.stream>>>(
        c.m, c.d_spins, c.d_bh, c.d_sweep, c.d_active, r.d_goff, r.d_box, r.d_slot, r.d_nbr,
        r.total_sites, r.d_bin_begin, r.d_bin_nred, r.d_bin_chain_begin, r.d_bin_chains, r.nbins,
        r.cap, nsweeps, fm);
}

template <int DIM, int DK, bool ISING, bool MEASURE>
int res_attr(size_t smem) {
    return cuda_check(cudaFuncSetAttribute(k_resident<DIM, DK, ISING, MEASURE>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                      "cudaFuncSetAttribute(k_resident)");
}

template <int DIM, bool ISING, bool MEASURE>
int set_attr_dk(int dk, size_t smem) {
    if (ISING) return res_attr<DIM, kDmiNone, true, MEASURE>(smem);
    switch (dk) {
        case kDmiNone: return res_attr<DIM, kDmiNone, false, MEASURE>(smem);
        case kDmiGeneral: return res_attr<DIM, kDmiGeneral, false, MEASURE>(smem);
        case kDmiPairs: return res_attr<DIM, kDmiPairs, false, MEASURE>(smem);
        default: return res_attr<DIM, kDmiAxial, false, MEASURE>(smem);
    }
}

int set_attr(Ctx& c, size_t smem) {
    const int dk = c.m.dmi_kind;
    if (c.dim == 3) return c.ising ? set_attr_dk<3, true, false>(dk, smem) : set_attr_dk<3, false, false>(dk, smem);
    int rc = c.ising ? set_attr_dk<2, true, false>(dk, smem) : set_attr_dk<2, false, false>(dk, smem);
    if (rc) return rc;
    return c.ising ? set_attr_dk<2, true, true>(dk, smem) : set_attr_dk<2, false, true>(dk, smem);
}

template <int DIM, bool ISING, bool MEASURE>
void launch_dk(Ctx& c, int grid, int nsweeps, const FusedMeasure& fm) {
    if (ISING) {
        res_launch<DIM, kDmiNone, true, MEASURE>(c, grid, nsweeps, fm);
        return;
    }
    switch (c.m.dmi_kind) {
        case kDmiNone: res_launch<DIM, kDmiNone, false, MEASURE>(c, grid, nsweeps, fm); break;
        case kDmiGeneral: res_launch<DIM, kDmiGeneral, false, MEASURE>(c, grid, nsweeps, fm); break;
        case kDmiPairs: res_launch<DIM, kDmiPairs, false, MEASURE>(c, grid, nsweeps, fm); break;
        default: res_launch<DIM, kDmiAxial, false, MEASURE>(c, grid, nsweeps, fm); break;
    }
}

void do_launch(Ctx& c, int grid, int nsweeps, const FusedMeasure* fm = nullptr) {
    const FusedMeasure none{};
    if (c.dim == 3) {
        if (c.ising) launch_dk<3, true, false>(c, grid, nsweeps, none);
        else launch_dk<3, false, false>(c, grid, nsweeps, none);
    } else if (fm) {
        if (c.ising) launch_dk<2, true, true>(c, grid, nsweeps, *fm);
        else launch_dk<2, false, true>(c, grid, nsweeps, *fm);
    } else {
        if (c.ising) launch_dk<2, true, false>(c, grid, nsweeps, none);
        else launch_dk<2, false, false>(c, grid, nsweeps, none);
    }
}

int grid_for(const Ctx& c) {
    // all bins resident at once when they fit; otherwise the CTAs loop over bins
    const ResidentTables& r = c.res;
    size_t smem = (size_t)r.cap * site_bytes(c) + 2048;
    int per_sm_smem = (int)std::max<size_t>(1, (c.smem_optin + 1024) / smem);
    int per_sm_thr = std::max(1, 2048 / r.threads);
    int per_sm = std::min(per_sm_smem, per_sm_thr);
    int cap_ctas = std::max(1, per_sm * c.sm_count);
    return std::min(r.nbins, cap_ctas);
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
    std::string g = c.gpu_name;
    for (char& ch : g)
        if (ch == ' ') ch = '_';
    char buf[64];
    snprintf(buf, sizeof buf, "%016llx", (unsigned long long)h);
    return g + ":" + buf;
}

bool cache_lookup(const std::string& key, int& nbins, int& threads) {
    std::ifstream f(cache_path());
    std::string k;
    int b, t;
    bool found = false;
    while (f >> k >> b >> t)
        if (k == key) {
            nbins = b;
            threads = t;
            found = true;
        }
    return found;
}

void cache_store(const std::string& key, int nbins, int threads) {
    std::ofstream f(cache_path(), std::ios::app);
    if (f) f << key << " " << nbins << " " << threads << "\n";
}

}  // namespace

void resident_free(Ctx& c) { free_tables(c.res); }

// Decides eligibility and builds the tables (autotuned unless options fix the shape).
int resident_prepare(Ctx& c) {
    if (c.res.built) return NMMC_OK;
    const size_t budget = smem_budget(c);
    const int cap_sites = (int)std::min<size_t>(65534, budget / site_bytes(c));
    int maxn = 0;
    for (int v : c.num) maxn = std::max(maxn, v);
    c.res.eligible = maxn > 0 && maxn <= cap_sites;
    if (!c.res.eligible) return NMMC_OK;

    std::vector<int> load(c.num.begin(), c.num.end());
    auto try_shape = [&](int nbins, int threads) -> int {
        std::vector<std::vector<int>> bins;
        if (!pack_bins(load, nbins, cap_sites, bins)) return NMMC_ERR_UNSUPPORTED;
        int rc = build_tables(c, bins, threads);
        if (rc) return rc;
        return set_attr(c, (size_t)c.res.cap * site_bytes(c));
    };

    int fixed_bins = c.res_bins, fixed_threads = c.res_threads;
    if (fixed_bins > 0 && fixed_threads > 0) return try_shape(std::min(fixed_bins, c.nchains), fixed_threads);

    // candidate shapes
    long total = std::accumulate(load.begin(), load.end(), 0L);
    int min_bins = (int)std::max<long>(1, (total + cap_sites - 1) / cap_sites);
    std::vector<int> cand_bins;
    for (int k : {1, 2, 3, 4}) cand_bins.push_back(std::min(c.nchains, std::max(min_bins, k * c.sm_count)));
    cand_bins.push_back(c.nchains);
    std::sort(cand_bins.begin(), cand_bins.end());
    cand_bins.erase(std::unique(cand_bins.begin(), cand_bins.end()), cand_bins.end());
    std::vector<int> cand_threads = {128, 256, 512, 1024};
    if (fixed_bins > 0) cand_bins = {std::min(fixed_bins, c.nchains)};
    if (fixed_threads > 0) cand_threads = {fixed_threads};

    const std::string key = config_key(c);
    int cb = 0, ct = 0;
    if (cache_lookup(key, cb, ct)) {
        if (try_shape(cb, ct) == NMMC_OK) return NMMC_OK;
    }

    // time each candidate on the live chains; spins and counters are restored afterwards
    void* snap = nullptr;
    unsigned long long* snap_sw = nullptr;
    NMMC_CUDA(cudaMalloc(&snap, c.spins_bytes));
    NMMC_CUDA(cudaMalloc(&snap_sw, sizeof(unsigned long long) * c.nchains));
    NMMC_CUDA(cudaMemcpyAsync(snap, c.d_spins, c.spins_bytes, cudaMemcpyDeviceToDevice, c.stream));
    NMMC_CUDA(cudaMemcpyAsync(snap_sw, c.d_sweep, sizeof(unsigned long long) * c.nchains,
                              cudaMemcpyDeviceToDevice, c.stream));
    NMMC_CUDA(cudaMemsetAsync(c.d_active, 1, c.nchains, c.stream));
    int rc = upload_params(c);
    if (rc) return rc;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    float best = 1e30f;
    int best_b = 0, best_t = 0;
    for (int nb : cand_bins)
        for (int th : cand_threads) {
            if (try_shape(nb, th) != NMMC_OK) continue;
            int grid = grid_for(c);
            do_launch(c, grid, 1);   // warm-up
            cudaEventRecord(a, c.stream);
            do_launch(c, grid, 8);
            cudaEventRecord(b, c.stream);
            if (cudaEventSynchronize(b) != cudaSuccess) break;
            float ms = 0;
            cudaEventElapsedTime(&ms, a, b);
            if (cudaGetLastError() != cudaSuccess) continue;
            if (ms < best) {
                best = ms;
                best_b = nb;
                best_t = th;
            }
        }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaMemcpyAsync(c.d_spins, snap, c.spins_bytes, cudaMemcpyDeviceToDevice, c.stream);
    cudaMemcpyAsync(c.d_sweep, snap_sw, sizeof(unsigned long long) * c.nchains, cudaMemcpyDeviceToDevice, c.stream);
    NMMC_CUDA(cudaStreamSynchronize(c.stream));
    cudaFree(snap);
    cudaFree(snap_sw);
    if (best_b == 0) {
        c.res.eligible = false;
        return NMMC_OK;
    }
    cache_store(key, best_b, best_t);
    return try_shape(best_b, best_t);
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
    if (measure) {
        if (!resident_can_measure(c)) return set_error(NMMC_ERR_UNSUPPORTED, "fused measurement not available");
        FusedMeasure fm{c.d_obs, c.d_q, c.d_acc, c.d_Hd, direct_all ? nullptr : c.d_pos,
                        c.res.d_slot_red, c.res.d_slot_black, accumulate};
        do_launch(c, grid_for(c), nsweeps, &fm);
    } else {
        do_launch(c, grid_for(c), nsweeps);
    }
    return cuda_check(cudaGetLastError(), "k_resident launch");
}

}  // namespace nmmc
