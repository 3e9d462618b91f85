// General interaction tables: any list of offsets with J and D per record, read as the
// reference reads them (Old/lib/field_type.cpp:49-71) and summed in file order like its
// neighbour lists (field_type.cpp:104-141, thermodynamics.cpp:17-69). Tables beyond the
// 2*dim axis neighbours (next-nearest, third-nearest, long-range exchange) cannot use the
// two-colour checkerboard, so the lattice is split into colour classes in which no two sites
// interact through any record (find_colouring, nmmc_host.cpp); one launch updates one class
// of every listed chain, gathering each site's neighbours record by record.
//
// The Philox draw of a site is the one the checkerboard kernels use (box index, sweep
// counter, chain), so only the order of the classes differs from them.
#include "nmmc_kernels.cuh"

namespace nmmc {

// Site handled by thread t of colour class `colour`; false when the thread has none.
template <int DIM>
__device__ __forceinline__ bool colour_site(const DevModel& m, int colour, int t, int& x, int& y, int& z) {
    if (m.col_kind == 1) {   // x + b*y + c*z = colour (mod q): x steps by q along each row
        const int q = m.col_q;
        const int kx = (m.edge + q - 1) / q;
        const int row = t / kx, k = t - row * kx;
        if (row >= m.ly * m.lz) return false;
        z = (DIM == 3) ? row / m.ly : 0;
        y = row - z * m.ly;
        int r = (colour - m.col_b * y - m.col_c * z) % q;
        if (r < 0) r += q;
        x = r + k * q;
    } else {                 // (x, y, z) = (cx, cy, cz) (mod p)
        const int p = m.col_p;
        const int cx = colour % p, cy = (colour / p) % p, cz = (DIM == 3) ? colour / (p * p) : 0;
        const int kx = (m.edge - cx + p - 1) / p, ky = (m.ly - cy + p - 1) / p;
        const int kz = (DIM == 3) ? (m.lz - cz + p - 1) / p : 1;
        const int k = t % kx, rest = t / kx;
        const int jy = rest % ky, jz = rest / ky;
        if (jz >= kz) return false;
        x = cx + k * p;
        y = cy + jy * p;
        z = cz + jz * p;
    }
    return x < m.edge;
}

// Neighbour of (x, y, z) through record offset o: its box coordinates, or false when it falls
// off an open boundary or is the site itself (the reference skips i == j). On periodic
// lattices the offsets are stored wrapped into [0, edge) and o.w marks a record that wraps
// onto the site itself, so the wrap is one conditional subtraction per axis.
template <int DIM, bool PERIODIC>
__device__ __forceinline__ bool general_neighbour(const DevModel& m, int x, int y, int z, int4 o, int& qx,
                                                  int& qy, int& qz) {
    qx = x + o.x;
    qy = y + o.y;
    qz = (DIM == 3) ? z + o.z : 0;
    if (PERIODIC) {
        const int e = m.edge;
        qx -= (qx >= e) ? e : 0;
        qy -= (qy >= e) ? e : 0;
        if (DIM == 3) qz -= (qz >= e) ? e : 0;
    } else {
        if (qx < 0 || qx >= m.edge || qy < 0 || qy >= m.edge) return false;
        if (DIM == 3 && (qz < 0 || qz >= m.edge)) return false;
    }
    return o.w == 0;
}

__device__ __forceinline__ size_t plane_index(const DevModel& m, int x, int y, int z) {
    return (size_t)(z * m.ly + y) * m.hx + (x >> 1);
}

// Records per batch of the gathers: the neighbour loads of kRecBatch records are issued
// before any of their terms is added, so their latencies overlap; the terms are still added
// one record at a time in file order.
constexpr int kRecBatch = 4;

// Local field of the sweep, FP32, records in file order: H + sum_r J_r s_r + s_r x Ds_r.
// Sites outside a particle hold 0 and add nothing. Ising: hx only.
template <int DIM, bool PERIODIC, bool ISING>
__device__ __forceinline__ void general_field(const DevModel& m, const void* __restrict__ spins_v, int chain,
                                              int x, int y, int z, float4 p, float& hx, float& hy, float& hz) {
    const size_t P = (size_t)m.nhalf_pad;
    const int8_t* si = (const int8_t*)spins_v + (size_t)chain * 2 * P;
    const float* sf = (const float*)spins_v + (size_t)chain * 2 * 3 * P;
    hx = p.y;
    hy = p.z;
    hz = p.w;
    const int ngen = m.ngen;
    for (int r0 = 0; r0 < ngen; r0 += kRecBatch) {
        float vx[kRecBatch], vy[kRecBatch], vz[kRecBatch];
        bool ok[kRecBatch];
#pragma unroll
        for (int u = 0; u < kRecBatch; ++u) {
            const int r = r0 + u;
            int qx, qy, qz;
            ok[u] = r < ngen && general_neighbour<DIM, PERIODIC>(m, x, y, z, __ldg(&m.g_off[r]), qx, qy, qz);
            vx[u] = vy[u] = vz[u] = 0.0f;
            if (ok[u]) {
                const size_t c2 = (size_t)((qx + qy + qz) & 1);
                const size_t j = plane_index(m, qx, qy, qz);
                if (ISING) {
                    vx[u] = (float)si[c2 * P + j];
                } else {
                    const float* pl = sf + c2 * 3 * P;
                    vx[u] = pl[j];
                    vy[u] = pl[P + j];
                    vz[u] = pl[2 * P + j];
                }
            }
        }
#pragma unroll
        for (int u = 0; u < kRecBatch; ++u) {
            if (!ok[u]) continue;
            const float4 js = __ldg(&m.g_js[r0 + u]);
            const float sx = vx[u], sy = vy[u], sz = vz[u];
            hx = fmaf(js.x, sx, hx);
            if (!ISING) {
                hy = fmaf(js.x, sy, hy);
                hz = fmaf(js.x, sz, hz);
                hx = fmaf(sy, js.w, fmaf(-sz, js.z, hx));   // s x Ds
                hy = fmaf(sz, js.y, fmaf(-sx, js.w, hy));
                hz = fmaf(sx, js.z, fmaf(-sy, js.y, hz));
            }
        }
    }
}

// One colour class of every listed chain (grid.y = list position).
template <int DIM, bool PERIODIC, bool MASKED, bool ISING>
__global__ void __launch_bounds__(256)
k_colour_sweep(const DevModel m, void* __restrict__ spins_v, const uint8_t* __restrict__ mask,
               const float4* __restrict__ bh, const unsigned long long* __restrict__ sweep,
               const int* __restrict__ chains, int colour, unsigned off) {
    const int chain = chains[blockIdx.y];
    int x, y, z;
    if (!colour_site<DIM>(m, colour, blockIdx.x * blockDim.x + threadIdx.x, x, y, z)) return;
    const int c2 = (x + y + z) & 1;
    const size_t P = (size_t)m.nhalf_pad;
    const size_t i = plane_index(m, x, y, z);
    if (MASKED && !mask[((size_t)chain * 2 + c2) * P + i]) return;
    const float4 p = bh[chain];
    const uint32_t box = (uint32_t)(x + m.edge * (y + m.edge * z));
    const nmmc_u4 r = sweep_draw(m, box, sweep[chain] + off, (uint32_t)chain);
    float hx, hy, hz;
    general_field<DIM, PERIODIC, ISING>(m, spins_v, chain, x, y, z, p, hx, hy, hz);
    if (ISING) {
        int8_t* own = (int8_t*)spins_v + ((size_t)chain * 2 + c2) * P + i;
        float t;
        if (ising_try(hx, (float)*own, p, r, t)) *own = (int8_t)t;
    } else {
        float* pl = (float*)spins_v + ((size_t)chain * 2 + c2) * 3 * P;
        float tx, ty, tz;
        if (heis_try(hx, hy, hz, pl[i], pl[P + i], pl[2 * P + i], p, r, tx, ty, tz)) {
            pl[i] = tx;
            pl[P + i] = ty;
            pl[2 * P + i] = tz;
        }
    }
}

// Threads per chain for one colour class (the largest class).
static int colour_threads(const Ctx& c) {
    const DevModel& m = c.m;
    if (m.col_kind == 1) return m.ly * m.lz * ((m.edge + m.col_q - 1) / m.col_q);
    const int k = (m.edge + m.col_p - 1) / m.col_p;
    return k * k * (c.dim == 3 ? k : 1);
}

template <int DIM, bool PERIODIC, bool MASKED, bool ISING>
static void colour_launch(Ctx& c, const int* d_chains, int n, int colour, unsigned off) {
    dim3 grid((colour_threads(c) + 255) / 256, n);
    k_colour_sweep<DIM, PERIODIC, MASKED, ISING><<<grid, 256, 0, c.stream>>>(
        c.m, c.d_spins, c.d_mask, c.d_bh, c.d_sweep, d_chains, colour, off);
}

using ColourFn = void (*)(Ctx&, const int*, int, int, unsigned);

template <int DIM, bool PERIODIC>
static ColourFn pick_colour_pm(const Ctx& c) {
    if (c.ising) return c.masked ? colour_launch<DIM, PERIODIC, true, true> : colour_launch<DIM, PERIODIC, false, true>;
    return c.masked ? colour_launch<DIM, PERIODIC, true, false> : colour_launch<DIM, PERIODIC, false, false>;
}

int launch_colour_sweeps(Ctx& c, const int* d_chains, int n, int nsweeps) {
    ColourFn f = (c.dim == 3) ? (c.periodic ? pick_colour_pm<3, true>(c) : pick_colour_pm<3, false>(c))
                              : (c.periodic ? pick_colour_pm<2, true>(c) : pick_colour_pm<2, false>(c));
    for (int s = 0; s < nsweeps; ++s)
        for (int colour = 0; colour < c.m.col_q; ++colour) f(c, d_chains, n, colour, (unsigned)s);
    int rc = cuda_check(cudaGetLastError(), "colour-sweep launch");
    if (rc) return rc;
    return launch_advance(c, d_chains, n, nsweeps);
}

// ------------------------------------------------------------------------------------------
// Energy term of a general table (thermodynamics.cpp:71-96): sum_i s_i . sum_r (J_r s_r +
// De_r x s_r), added to slot 0 of the partial sums the measurement kernel wrote for the same
// blocks (same rows-per-block split), so the finalisation is unchanged.
// ------------------------------------------------------------------------------------------
template <int DIM, bool PERIODIC, bool MASKED, bool ISING, typename RT>
__global__ void __launch_bounds__(256)
k_energy_general(const DevModel m, const void* __restrict__ spins_v, const uint8_t* __restrict__ mask,
                 const int* __restrict__ chains, int rows, int nblk_slice, int nblk_total,
                 double* __restrict__ partial) {
    const int ci = blockIdx.y;
    const int chain = chains[ci];
    const int b = blockIdx.x;
    const int z = b / nblk_slice;
    const int y0 = (b - z * nblk_slice) * rows;
    const int y1 = min(y0 + rows, m.ly);
    const int nsite = (y1 - y0) * m.edge;
    const size_t P = (size_t)m.nhalf_pad;
    auto load = [&](int x, int y, int zz, RT& s0, RT& s1, RT& s2) {
        const int c2 = (x + y + zz) & 1;
        const size_t i = plane_index(m, x, y, zz);
        if (ISING) {
            s0 = RT(((const int8_t*)spins_v)[((size_t)chain * 2 + c2) * P + i]);
            s1 = s2 = RT(0);
        } else {
            const float* pl = (const float*)spins_v + ((size_t)chain * 2 + c2) * 3 * P;
            s0 = RT(pl[i]);
            s1 = RT(pl[P + i]);
            s2 = RT(pl[2 * P + i]);
        }
    };
    RT acc = RT(0);
    for (int t = threadIdx.x; t < nsite; t += blockDim.x) {
        const int yy = t / m.edge, y = y0 + yy, x = t - yy * m.edge;
        if (MASKED && !mask[((size_t)chain * 2 + ((x + y + z) & 1)) * P + plane_index(m, x, y, z)]) continue;
        RT s0, s1, s2;
        load(x, y, z, s0, s1, s2);
        RT f0 = RT(0), f1 = RT(0), f2 = RT(0);
        const int ngen = m.ngen;
        for (int r0 = 0; r0 < ngen; r0 += kRecBatch) {
            RT a0[kRecBatch], a1[kRecBatch], a2[kRecBatch];
            bool ok[kRecBatch];
#pragma unroll
            for (int u = 0; u < kRecBatch; ++u) {   // loads of the batch first, terms in file order
                const int r = r0 + u;
                int qx, qy, qz;
                ok[u] = r < ngen && general_neighbour<DIM, PERIODIC>(m, x, y, z, __ldg(&m.g_off[r]), qx, qy, qz);
                a0[u] = a1[u] = a2[u] = RT(0);
                if (ok[u]) load(qx, qy, qz, a0[u], a1[u], a2[u]);
            }
#pragma unroll
            for (int u = 0; u < kRecBatch; ++u) {
                if (!ok[u]) continue;
                const int r = r0 + u;
                const RT n0 = a0[u], n1 = a1[u], n2 = a2[u];
                RT J, d0, d1, d2;
                if (sizeof(RT) == 8) {
                    J = RT(m.g_jed[4 * r]);
                    d0 = RT(m.g_jed[4 * r + 1]);
                    d1 = RT(m.g_jed[4 * r + 2]);
                    d2 = RT(m.g_jed[4 * r + 3]);
                } else {
                    const float4 je = __ldg(&m.g_je[r]);
                    J = RT(je.x);
                    d0 = RT(je.y);
                    d1 = RT(je.z);
                    d2 = RT(je.w);
                }
                f0 += J * n0;
                if (!ISING) {
                    f1 += J * n1;
                    f2 += J * n2;
                    f0 += d1 * n2 - d2 * n1;   // De x s_j
                    f1 += d2 * n0 - d0 * n2;
                    f2 += d0 * n1 - d1 * n0;
                }
            }
        }
        acc += s0 * f0 + s1 * f1 + s2 * f2;
    }
    // warp sums in the mode's type (FP32 mode: as the measurement kernels), FP64 across warps
    __shared__ RT red[8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    RT v = acc;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double tot = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += (double)red[w];
        partial[((size_t)ci * nblk_total + b) * kNP] += tot;
    }
}

template <int DIM, bool PERIODIC, bool MASKED, bool ISING>
static void energy_launch(Ctx& c, const int* d_chains, int n, int rows, int nblk_slice, int nblk_total,
                          double* partial) {
    dim3 grid(nblk_slice * c.m.lz, n);
    if (c.measure_fp64)
        k_energy_general<DIM, PERIODIC, MASKED, ISING, double><<<grid, 256, 0, c.stream>>>(
            c.m, c.d_spins, c.d_mask, d_chains, rows, nblk_slice, nblk_total, partial);
    else
        k_energy_general<DIM, PERIODIC, MASKED, ISING, float><<<grid, 256, 0, c.stream>>>(
            c.m, c.d_spins, c.d_mask, d_chains, rows, nblk_slice, nblk_total, partial);
}

template <int DIM, bool PERIODIC>
static void energy_pm(Ctx& c, const int* d, int n, int rows, int nbs, int nbt, double* partial) {
    if (c.ising) {
        if (c.masked) energy_launch<DIM, PERIODIC, true, true>(c, d, n, rows, nbs, nbt, partial);
        else energy_launch<DIM, PERIODIC, false, true>(c, d, n, rows, nbs, nbt, partial);
    } else {
        if (c.masked) energy_launch<DIM, PERIODIC, true, false>(c, d, n, rows, nbs, nbt, partial);
        else energy_launch<DIM, PERIODIC, false, false>(c, d, n, rows, nbs, nbt, partial);
    }
}

int launch_energy_general(Ctx& c, const int* d_chains, int n, int rows, int nblk_slice, int nblk_total,
                          double* partial) {
    if (c.dim == 3) {
        if (c.periodic) energy_pm<3, true>(c, d_chains, n, rows, nblk_slice, nblk_total, partial);
        else energy_pm<3, false>(c, d_chains, n, rows, nblk_slice, nblk_total, partial);
    } else {
        if (c.periodic) energy_pm<2, true>(c, d_chains, n, rows, nblk_slice, nblk_total, partial);
        else energy_pm<2, false>(c, d_chains, n, rows, nblk_slice, nblk_total, partial);
    }
    return cuda_check(cudaGetLastError(), "k_energy_general");
}

// ------------------------------------------------------------------------------------------
// dE probe with the general sweep's FP32 field.
// ------------------------------------------------------------------------------------------
template <int DIM, bool PERIODIC, bool ISING>
__global__ void k_delta_e_general(const DevModel m, const void* __restrict__ spins_v,
                                  const float4* __restrict__ bh, int chain, const int32_t* __restrict__ sites,
                                  const float* __restrict__ trial, int n, double* __restrict__ out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int box = sites[t];
    const int x = box % m.edge, y = (box / m.edge) % m.edge, z = (DIM == 3) ? box / (m.edge * m.edge) : 0;
    const int c2 = (x + y + z) & 1;
    const size_t P = (size_t)m.nhalf_pad, i = plane_index(m, x, y, z);
    float hx, hy, hz;
    general_field<DIM, PERIODIC, ISING>(m, spins_v, chain, x, y, z, bh[chain], hx, hy, hz);
    if (ISING) {
        const float so = (float)((const int8_t*)spins_v)[((size_t)chain * 2 + c2) * P + i];
        out[t] = (double)(hx * (so - trial[3 * t]));
    } else {
        const float* pl = (const float*)spins_v + ((size_t)chain * 2 + c2) * 3 * P;
        out[t] = (double)heis_dE(hx, hy, hz, pl[i], pl[P + i], pl[2 * P + i], trial[3 * t], trial[3 * t + 1],
                                 trial[3 * t + 2]);
    }
}

int launch_delta_e_general(Ctx& c, int chain, const int32_t* d_sites, const float* d_trial, int n, double* d_out) {
    const int g = (n + 127) / 128;
#define NMMC_DEG(D, PR, IS) \
    k_delta_e_general<D, PR, IS><<<g, 128, 0, c.stream>>>(c.m, c.d_spins, c.d_bh, chain, d_sites, d_trial, n, d_out)
    if (c.dim == 3) {
        if (c.periodic) { if (c.ising) NMMC_DEG(3, true, true); else NMMC_DEG(3, true, false); }
        else { if (c.ising) NMMC_DEG(3, false, true); else NMMC_DEG(3, false, false); }
    } else {
        if (c.periodic) { if (c.ising) NMMC_DEG(2, true, true); else NMMC_DEG(2, true, false); }
        else { if (c.ising) NMMC_DEG(2, false, true); else NMMC_DEG(2, false, false); }
    }
#undef NMMC_DEG
    return cuda_check(cudaGetLastError(), "k_delta_e_general");
}

// ------------------------------------------------------------------------------------------
// Device records
// ------------------------------------------------------------------------------------------
int upload_general(Ctx& c) {
    const size_t n = c.h_gje.size();
    if (!n) return NMMC_OK;
    std::vector<float4> js(n);
    for (size_t r = 0; r < n; ++r) {   // sweep convention: s_j x D (reference) or D x s_j
        const float4& e = c.h_gje[r];
        js[r] = c.dmi_sign ? make_float4(e.x, -e.y, -e.z, -e.w) : e;
    }
    NMMC_CUDA(cudaMemcpyAsync(c.d_gjs, js.data(), n * sizeof(float4), cudaMemcpyHostToDevice, c.stream));
    return cuda_check(cudaStreamSynchronize(c.stream), "upload_general");
}

}  // namespace nmmc
