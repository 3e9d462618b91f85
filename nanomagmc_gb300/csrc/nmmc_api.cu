// C ABI of libnmmc: context lifecycle, chain parameters, sweeps, observables, graphs,
// spin I/O and the parity probes. See include/nmmc.h for the contract of each call.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "nmmc_internal.h"

struct nmmc_ctx : public nmmc::Ctx {};

namespace nmmc {

int cuda_check(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return NMMC_OK;
    return set_error(NMMC_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

void classify_dmi(DevModel& m) {
    if (!m.has_dmi) {
        m.dmi_kind = 0;   // kDmiNone
        return;
    }
    bool pairs = true, axial = true;
    for (int a = 0; a < m.dim; ++a) {
        const int kp = 2 * a, km = 2 * a + 1;
        if (m.J[kp] != m.J[km]) pairs = false;
        for (int c = 0; c < 3; ++c) {
            if (m.Ds[kp][c] != -m.Ds[km][c]) pairs = false;
            if (c != a && m.Ds[kp][c] != 0.0f) axial = false;
        }
    }
    m.dmi_kind = !pairs ? 1 : (axial ? 3 : 2);   // kDmiGeneral / kDmiAxial / kDmiPairs
}

// (beta, H) of every chain to the device, through the context's pinned staging buffers.
int upload_params(Ctx& c) {
    if (!c.params_dirty) return NMMC_OK;
    NMMC_CUDA(cudaEventSynchronize(c.ev_params));   // the previous upload has left the staging
    const int hi = c.ising ? 0 : 2;   // h_ind (Old/lib/state.cpp:22-28)
    for (int i = 0; i < c.nchains; ++i) {
        double beta = 1.0 / (c.k_b * c.T[i]);
        float H[3] = {0, 0, 0};
        H[hi] = (float)c.H[i];
        c.h_bh[i] = make_float4((float)beta, H[0], H[1], H[2]);
        for (int k = 0; k < 3; ++k) c.h_hd[3 * (size_t)i + k] = (k == hi) ? c.H[i] : 0.0;
    }
    // (beta, H) and the FP64 fields are one contiguous block on both sides: one copy
    NMMC_CUDA(cudaMemcpyAsync(c.d_bh, c.h_bh, (sizeof(float4) + 3 * sizeof(double)) * c.nchains,
                              cudaMemcpyHostToDevice, c.stream));
    NMMC_CUDA(cudaEventRecord(c.ev_params, c.stream));
    c.params_dirty = false;
    return NMMC_OK;
}

// A list that names every chain in order is the all-chains call: no list upload, and the
// resident path keeps its chain marks.
static const int* all_if_identity(const Ctx& c, const int* chains, int n) {
    if (!chains || n != c.nchains) return chains;
    for (int i = 0; i < n; ++i)
        if (chains[i] != i) return chains;
    return nullptr;
}

// Chain list checks shared by every call that takes one: indices in range, none listed twice
// (two entries of one chain would update it from two blocks at once, or add its sample twice).
static int check_list(Ctx& c, const int* chains, int n) {
    if (n < 0 || n > c.nchains) return set_error(NMMC_ERR_ARG, "chain count %d out of range", n);
    c.list_seen.assign((size_t)c.nchains, 0);
    for (int i = 0; i < n; ++i) {
        if (chains[i] < 0 || chains[i] >= c.nchains)
            return set_error(NMMC_ERR_ARG, "chain index %d out of range", chains[i]);
        if (c.list_seen[chains[i]]++) return set_error(NMMC_ERR_ARG, "chain %d listed twice", chains[i]);
    }
    return NMMC_OK;
}

static int set_list(Ctx& c, const int* chains, int n, const int** d_out) {
    if (!chains) {
        *d_out = c.d_all;
        return NMMC_OK;
    }
    if (int rc = check_list(c, chains, n)) return rc;
    // through the pinned staging buffer: the caller's array is read before the call returns
    NMMC_CUDA(cudaEventSynchronize(c.ev_list));
    memcpy(c.h_list, chains, sizeof(int) * n);
    NMMC_CUDA(cudaMemcpyAsync(c.d_list, c.h_list, sizeof(int) * n, cudaMemcpyHostToDevice, c.stream));
    NMMC_CUDA(cudaEventRecord(c.ev_list, c.stream));
    *d_out = c.d_list;
    return NMMC_OK;
}

static bool use_resident(Ctx& c, int* rc) {
    *rc = NMMC_OK;
    if (c.sweep_path == 1) return false;
    *rc = resident_prepare(c);
    if (*rc) return false;
    if (c.sweep_path == 2 && !c.res.eligible) {
        *rc = set_error(NMMC_ERR_UNSUPPORTED, "lattice does not fit the shared-memory resident path");
        return false;
    }
    return resident_chosen(c);
}

long long count_sites(const Ctx& c, const int* h_chains, int n) {
    long long sites = 0;
    if (!h_chains) {
        for (int v : c.num) sites += v;
    } else {
        for (int i = 0; i < n; ++i) sites += c.num[h_chains[i]];
    }
    return sites;
}

// Sweep-kernel timing: event pairs are recorded around each sweep call and resolved when
// the totals are read, so timing never synchronises the stream between calls.
static int timing_begin(Ctx& c, TimedCall& t) {
    if (!c.ev_pool.empty()) {
        t.a = c.ev_pool.back().a;
        t.b = c.ev_pool.back().b;
        c.ev_pool.pop_back();
    } else {
        NMMC_CUDA(cudaEventCreate(&t.a));
        NMMC_CUDA(cudaEventCreate(&t.b));
    }
    NMMC_CUDA(cudaEventRecord(t.a, c.stream));
    return NMMC_OK;
}

int resolve_timing(Ctx& c) {
    for (TimedCall& t : c.pending) {
        NMMC_CUDA(cudaEventSynchronize(t.b));
        float ms = 0;
        NMMC_CUDA(cudaEventElapsedTime(&ms, t.a, t.b));
        c.t_ms += ms;
        c.t_launches += t.launches;
        c.t_updates += t.updates;
        c.ev_pool.push_back(t);
    }
    c.pending.clear();
    return NMMC_OK;
}

// Sweeps (and, with `fused`, the resident kernel's observables) of the listed chains, with
// optional event timing around the launch.
static int run_sweeps(Ctx& c, const int* d_chains, const int* h_chains, int n, int nsweeps, bool res,
                      bool fused, int accumulate, bool allow_timing) {
    const bool timed = allow_timing && c.timing;
    TimedCall t{};
    int rc;
    if (timed && (rc = timing_begin(c, t))) return rc;
    rc = res ? launch_resident_sweeps(c, d_chains, n, nsweeps, h_chains == nullptr, fused, accumulate)
         : c.m.general ? launch_colour_sweeps(c, d_chains, n, nsweeps)
                       : launch_global_sweeps(c, d_chains, n, nsweeps, fused);
    if (rc) return rc;
    if (timed) {
        NMMC_CUDA(cudaEventRecord(t.b, c.stream));
        t.launches = res ? resident_launches(c, nsweeps) : global_sweep_launches(c, nsweeps, fused);
        t.updates = count_sites(c, h_chains, n) * nsweeps;
        c.pending.push_back(t);
    }
    return NMMC_OK;
}

int sweep_impl(Ctx& c, const int* d_chains, const int* h_chains, int n, int nsweeps, bool allow_timing) {
    if (nsweeps <= 0 || n == 0) return NMMC_OK;
    int rc = upload_params(c);
    if (rc) return rc;
    bool res = use_resident(c, &rc);
    if (rc) return rc;
    return run_sweeps(c, d_chains, h_chains, n, nsweeps, res, false, 0, allow_timing);
}

// nsweeps sweeps, then the observables of the listed chains. On the resident path of a 2-D
// lattice both happen in one launch (the spins never leave shared memory); otherwise this is
// sweep_impl followed by launch_measure.
int sweep_measure_impl(Ctx& c, const int* d_chains, const int* h_chains, int n, int nsweeps, int accumulate,
                       bool allow_timing) {
    if (n == 0) return NMMC_OK;
    int rc = upload_params(c);
    if (rc) return rc;
    if (nsweeps > 0) {
        bool res = use_resident(c, &rc);
        if (rc) return rc;
        if (res && resident_can_measure(c)) {
            if ((rc = run_sweeps(c, d_chains, h_chains, n, nsweeps, true, true, accumulate, allow_timing))) return rc;
            return accumulate ? launch_add_av(c) : NMMC_OK;
        }
        if (!res && !c.m.general && hbm_fused_measure_ok(c)) {
            // E, M, subM and sub4M summed in the last colour-1 half-sweep, then the charge pass
            if ((rc = measure_prepare(c, n))) return rc;   // allocates only when the scratch is too small
            if ((rc = run_sweeps(c, d_chains, h_chains, n, nsweeps, false, true, 0, allow_timing))) return rc;
            if ((rc = launch_measure_fused_tail(c, d_chains, n, accumulate))) return rc;
            return accumulate ? launch_add_av(c) : NMMC_OK;
        }
        if ((rc = run_sweeps(c, d_chains, h_chains, n, nsweeps, res, false, 0, allow_timing))) return rc;
    }
    if ((rc = launch_measure(c, d_chains, n, accumulate))) return rc;
    return accumulate ? launch_add_av(c) : NMMC_OK;
}

static void destroy_ctx(Ctx* c) {
    if (!c) return;
    resident_free(*c);
    cudaFree(c->d_spins);
    cudaFree(c->d_spins_alt);
    cudaFree(c->d_mask);
    cudaFree(c->d_fill);
    cudaFree(c->d_fill_n);
    cudaFree(c->d_fill_zoff);
    cudaFree(c->d_cspins);
    cudaFree(c->d_ctab);
    cudaFree(c->d_bh);   // d_Hd lives in the same block
    cudaFree(c->d_sweep);
    cudaFree(c->d_all);
    cudaFree(c->d_list);
    cudaFree(c->d_active);
    cudaFree(c->d_pos);
    cudaFree(c->d_rm);
    cudaFreeHost(c->h_bh);   // h_hd lives in the same block
    cudaFreeHost(c->h_list);
    if (c->ev_params) cudaEventDestroy(c->ev_params);
    if (c->ev_list) cudaEventDestroy(c->ev_list);
    cudaFree(c->d_av);
    cudaFree(c->d_av_list);
    cudaFree(c->d_goff);
    cudaFree(c->d_gjs);
    cudaFree(c->d_gje);
    cudaFree(c->d_gjed);
    cudaFree(c->d_partial);
    cudaFree(c->d_mrows);
    cudaFree(c->d_obs);
    cudaFree(c->d_q);
    cudaFree(c->d_acc);
    cudaFree(c->d_replay);
    cudaFree(c->d_flag);
    for (TimedCall& t : c->pending) c->ev_pool.push_back(t);
    for (TimedCall& t : c->ev_pool) {
        cudaEventDestroy(t.a);
        cudaEventDestroy(t.b);
    }
    for (cudaEvent_t& e : c->marks)
        if (e) cudaEventDestroy(e);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete static_cast<nmmc_ctx*>(c);
}

// host <-> split-colour plane conversion for one chain
static void box_to_planes(const Ctx& c, const double* xyz, const uint8_t* mk, void* planes) {
    const int E = c.edge, nz = c.m.lz;
    const size_t P = (size_t)c.m.nhalf_pad;
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < E; ++y)
            for (int x = 0; x < E; ++x) {
                long box = x + (long)E * (y + (long)E * z);
                int colour = (x + y + z) & 1;
                size_t i = (size_t)(z * c.m.ly + y) * c.m.hx + (x >> 1);
                bool fill = !mk || mk[box];
                if (c.ising) {
                    double v = fill ? xyz[3 * box] : 0.0;
                    ((int8_t*)planes)[colour * P + i] = (int8_t)(v > 0 ? 1 : (v < 0 ? -1 : 0));
                } else {
                    float* f = (float*)planes + colour * 3 * P;
                    for (int k = 0; k < 3; ++k) f[k * P + i] = fill ? (float)xyz[3 * box + k] : 0.0f;
                }
            }
}

static void planes_to_box(const Ctx& c, const void* planes, double* xyz) {
    const int E = c.edge, nz = c.m.lz;
    const size_t P = (size_t)c.m.nhalf_pad;
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < E; ++y)
            for (int x = 0; x < E; ++x) {
                long box = x + (long)E * (y + (long)E * z);
                int colour = (x + y + z) & 1;
                size_t i = (size_t)(z * c.m.ly + y) * c.m.hx + (x >> 1);
                if (c.ising) {
                    xyz[3 * box] = ((const int8_t*)planes)[colour * P + i];
                    xyz[3 * box + 1] = xyz[3 * box + 2] = 0.0;
                } else {
                    const float* f = (const float*)planes + colour * 3 * P;
                    for (int k = 0; k < 3; ++k) xyz[3 * box + k] = f[k * P + i];
                }
            }
}

static size_t chain_elems(const Ctx& c) { return (size_t)2 * (c.ising ? 1 : 3) * c.m.nhalf_pad; }
static size_t elem_bytes(const Ctx& c) { return c.ising ? 1 : 4; }

// Mask planes of one chain, and its lists of filled sites per colour (compact indices in
// increasing order: z, y, then x), from the host mask.
static int upload_mask_chain(Ctx& c, int chain) {
    if (!c.masked) return NMMC_OK;
    const int E = c.edge, nz = c.m.lz;
    const size_t P = (size_t)c.m.nhalf_pad, NH = (size_t)c.m.nhalf;
    std::vector<uint8_t> pl(2 * P, 0);
    std::vector<uint32_t> fill[2];
    const uint8_t* mk = &c.mask[(size_t)chain * c.box_sites];
    int* zoff = &c.fill_zoff[(size_t)chain * 2 * (nz + 1)];   // colour 0 row, then colour 1
    for (int z = 0; z < nz; ++z) {
        zoff[z] = (int)fill[0].size();
        zoff[nz + 1 + z] = (int)fill[1].size();
        for (int y = 0; y < E; ++y)
            for (int x = 0; x < E; ++x) {
                long box = x + (long)E * (y + (long)E * z);
                int colour = (x + y + z) & 1;
                size_t i = (size_t)(z * c.m.ly + y) * c.m.hx + (x >> 1);
                pl[colour * P + i] = mk[box];
                if (mk[box]) fill[colour].push_back((uint32_t)i);
            }
    }
    zoff[nz] = (int)fill[0].size();
    zoff[nz + 1 + nz] = (int)fill[1].size();
    NMMC_CUDA(cudaMemcpy(c.d_mask + (size_t)chain * 2 * P, pl.data(), 2 * P, cudaMemcpyHostToDevice));
    NMMC_CUDA(cudaMemcpy(c.d_fill_zoff + (size_t)chain * 2 * (nz + 1), zoff, 2 * (nz + 1) * sizeof(int),
                         cudaMemcpyHostToDevice));
    for (int colour = 0; colour < 2; ++colour) {
        const int seg = chain * 2 + colour;
        if (fill[colour].size() > NH) return set_error(NMMC_ERR_ARG, "filled-site list longer than a colour plane");
        if (!fill[colour].empty())
            NMMC_CUDA(cudaMemcpy(c.d_fill + seg * NH, fill[colour].data(), fill[colour].size() * sizeof(uint32_t),
                                 cudaMemcpyHostToDevice));
        c.fill_n[seg] = (int)fill[colour].size();
    }
    NMMC_CUDA(cudaMemcpy(c.d_fill_n + chain * 2, &c.fill_n[chain * 2], 2 * sizeof(int), cudaMemcpyHostToDevice));
    c.fill_max = *std::max_element(c.fill_n.begin(), c.fill_n.end());
    int smax = 0;
    for (int ch = 0; ch < c.nchains; ++ch) {
        const int* zo = &c.fill_zoff[(size_t)ch * 2 * (nz + 1)];
        for (int z = 0; z < nz; ++z)
            smax = std::max(smax, (zo[z + 1] - zo[z]) + (zo[nz + 1 + z + 1] - zo[nz + 1 + z]));
    }
    c.fill_slice_max = smax;
    if (!c.ctab_built) return NMMC_OK;
    const int rc = compact_table_chain(c, chain);
    if (rc == kTableDoesNotFit) c.ctab_built = false;   // outgrew the packed table: rebuilt at the next sweep
    return rc == kTableDoesNotFit ? NMMC_OK : rc;
}

}  // namespace nmmc

using namespace nmmc;

extern "C" {

int nmmc_create(const nmmc_options* opt, const nmmc_interactions* inter, const nmmc_chain_desc* chains,
                int nchains, uint64_t seed, nmmc_ctx** out) {
    if (!opt || !inter || !chains || !out || nchains <= 0) return set_error(NMMC_ERR_ARG, "bad argument to nmmc_create");
    *out = nullptr;
    if (nchains > NMMC_MAX_CHAINS)
        return set_error(NMMC_ERR_ARG, "%d chains: at most %d per context", nchains, NMMC_MAX_CHAINS);
    const int dim = shape_dim(opt->shape_code);
    if (!dim) return set_error(NMMC_ERR_SHAPE, "Incorrect shape code '%c'", opt->shape_code);
    const int edge = (int)opt->edge_size;
    if (edge < 2) return set_error(NMMC_ERR_ARG, "lattice edge %d is below 2", edge);
    if (opt->k_b <= 0) return set_error(NMMC_ERR_TEMP, "Invalid Boltzmann constant");
    for (int i = 0; i < nchains; ++i)
        if (!(chains[i].T > 0)) return set_error(NMMC_ERR_TEMP, "Invalid temperature, chain %d", i);
    if (opt->is_perio && (edge & 1))
        return set_error(NMMC_ERR_UNSUPPORTED, "periodic lattices need an even edge for the checkerboard (edge %d)", edge);
    if (inter->dim != 0 && inter->dim != dim)
        return set_error(NMMC_ERR_ARG, "interaction table read for dim %d, lattice has dim %d", inter->dim, dim);
    if (inter->n < 0 || inter->n > NMMC_MAX_OFFSETS) return set_error(NMMC_ERR_ARG, "bad interaction record count");
    double Jdir[6], Ddir[6][3];
    std::string why;
    bool general = false;
    int rc = map_interactions(*inter, dim, opt->is_ising != 0, Jdir, Ddir, general, why);
    if (rc) return set_error_host(rc, why);
    Colouring col;
    if (general && (rc = find_colouring(*inter, dim, edge, opt->is_perio != 0, opt->is_ising != 0, col, why)))
        return set_error_host(rc, why);
    long long box = 1;
    for (int k = 0; k < dim; ++k) box *= edge;
    if (box > (1LL << 31)) return set_error(NMMC_ERR_UNSUPPORTED, "lattice box too large");

    nmmc_ctx* c = new nmmc_ctx();
    c->dim = dim;
    c->edge = edge;
    c->nchains = nchains;
    c->nslices = (dim == 3) ? edge : 1;
    c->box_sites = box;
    c->ising = opt->is_ising != 0;
    c->periodic = opt->is_perio != 0;
    c->shape = opt->shape_code;
    c->k_b = opt->k_b;
    c->seed = seed;
    c->inter = *inter;
    const bool weib = shape_is_weibull(opt->shape_code);
    c->masked = weib || (edge & 1);
    for (int i = 0; i < nchains; ++i) {
        c->T.push_back(chains[i].T);
        c->H.push_back(chains[i].H);
        c->size.push_back(chains[i].size);
    }
    const bool useJ = opt->J != 0, useD = opt->K != 0;   // Old/lib/state.cpp:17
    DevModel& m = c->m;
    m.dim = dim;
    m.edge = edge;
    m.lx = edge + (edge & 1);
    m.ly = edge;
    m.lz = (dim == 3) ? edge : 1;
    m.hx = m.lx / 2;
    m.nhalf = m.hx * m.ly * m.lz;
    m.nhalf_pad = (m.nhalf + 63) / 64 * 64;
    m.periodic = c->periodic;
    m.ising = c->ising;
    m.masked = c->masked;
    m.ndir = 2 * dim;
    m.has_dmi = 0;
    for (int k = 0; k < 6; ++k) {
        double J = useJ ? Jdir[k] : 0.0;
        m.J[k] = (float)J;
        m.Jd[k] = J;
        for (int a = 0; a < 3; ++a) {
            double D = (useD && !c->ising) ? Ddir[k][a] : 0.0;
            m.De[k][a] = (float)D;
            m.Ded[k][a] = D;
            m.Ds[k][a] = (float)D;   // dmi_sign 0: s_j x D
            if (D != 0) m.has_dmi = 1;
        }
    }
    classify_dmi(m);
    c->col = col;
    m.general = general ? 1 : 0;
    m.col_kind = col.kind;
    m.col_q = col.q;
    m.col_p = col.p;
    m.col_b = col.b;
    m.col_c = col.c;
    std::vector<int4> goff;
    std::vector<double> gjed;
    if (general) {
        // coupling records in file order (zero records and self-offsets add nothing)
        for (int r = 0; r < inter->n; ++r) {
            const int* o = inter->offset[r];
            if (o[0] == 0 && o[1] == 0 && (dim == 2 || o[2] == 0)) continue;
            const double J = useJ ? inter->J[r] : 0.0;
            double D[3];
            for (int a = 0; a < 3; ++a) D[a] = (useD && !c->ising) ? inter->D[r][a] : 0.0;
            if (J == 0 && D[0] == 0 && D[1] == 0 && D[2] == 0) continue;
            // periodic lattices: offsets wrapped into [0, edge) once here, so a kernel wraps with
            // one conditional subtraction; w = 1 marks a record that lands on the site itself
            // after the wrap (the reference skips i == j)
            int4 g = make_int4(o[0], o[1], dim == 3 ? o[2] : 0, 0);
            if (c->periodic) {
                const int e = m.edge;
                g.x = ((g.x % e) + e) % e;
                g.y = ((g.y % e) + e) % e;
                g.z = dim == 3 ? ((g.z % e) + e) % e : 0;
                g.w = (g.x == 0 && g.y == 0 && g.z == 0) ? 1 : 0;
            }
            goff.push_back(g);
            c->h_gje.push_back(make_float4((float)J, (float)D[0], (float)D[1], (float)D[2]));
            gjed.insert(gjed.end(), {J, D[0], D[1], D[2]});
        }
        m.ngen = (int)goff.size();
    }
    auto log2_or = [](int v) {
        if (v <= 0 || (v & (v - 1))) return -1;
        int k = 0;
        while ((1 << k) < v) ++k;
        return k;
    };
    m.qpr_shift = (m.hx % 4 == 0) ? log2_or(m.hx / 4) : -1;
    m.ly_shift = log2_or(m.ly);
    m.key0 = (uint32_t)seed;
    m.key1 = (uint32_t)(seed >> 32);
    for (int r = 0; r < 10; ++r) {
        m.rk0[r] = m.key0 + (uint32_t)r * 0x9E3779B9u;
        m.rk1[r] = m.key1 + (uint32_t)r * 0xBB67AE85u;
    }
    ReplayModel& r = c->rm;
    r.n = inter->n;
    for (int k = 0; k < inter->n; ++k) {
        for (int a = 0; a < 3; ++a) {
            r.off[k][a] = inter->offset[k][a];
            r.D[k][a] = inter->D[k][a];
        }
        r.J[k] = inter->J[k];
    }
    r.useJ = useJ;
    r.useD = useD && !c->ising;
    r.dmi_sign = 0;

    // shapes and site counts
    c->mask.assign((size_t)nchains * box, 1);
    c->num.resize(nchains);
    c->snum.resize(nchains);
    c->s4num.resize(nchains);
    for (int i = 0; i < nchains; ++i) {
        uint8_t* mk = &c->mask[(size_t)i * box];
        if (weib) {
            if (!(opt->beta_w > 0)) {
                destroy_ctx(c);
                return set_error(NMMC_ERR_ARG, "WEIBULLFACT must be positive");
            }
            weibull_mask(dim, edge, chains[i].size, opt->beta_w, seed, (uint32_t)chains[i].lattice, mk);
        }
        site_counts(dim, edge, weib ? mk : nullptr, &c->num[i], &c->snum[i], &c->s4num[i]);
    }

    // device
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    cudaDeviceProp prop;
    if (e == cudaSuccess) e = cudaGetDeviceProperties(&prop, dev);
    if (e != cudaSuccess) {
        destroy_ctx(c);
        return cuda_check(e, "cudaGetDeviceProperties");
    }
    c->device = dev;
    c->sm_count = prop.multiProcessorCount;
    c->smem_optin = prop.sharedMemPerBlockOptin;
    c->gpu_name = prop.name;
#define NMMC_TRY(call)                      \
    do {                                    \
        cudaError_t _e = (call);            \
        if (_e != cudaSuccess) {            \
            int _rc = cuda_check(_e, #call); \
            destroy_ctx(c);                 \
            return _rc;                     \
        }                                   \
    } while (0)
    NMMC_TRY(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    c->spins_bytes = chain_elems(*c) * elem_bytes(*c) * nchains;
    NMMC_TRY(cudaMalloc(&c->d_spins, c->spins_bytes));
    if (c->masked) {
        NMMC_TRY(cudaMalloc(&c->d_mask, (size_t)nchains * 2 * m.nhalf_pad));
        NMMC_TRY(cudaMemset(c->d_mask, 0, (size_t)nchains * 2 * m.nhalf_pad));
        NMMC_TRY(cudaMalloc(&c->d_fill, (size_t)nchains * 2 * m.nhalf * sizeof(uint32_t)));
        NMMC_TRY(cudaMalloc(&c->d_fill_n, (size_t)nchains * 2 * sizeof(int)));
        NMMC_TRY(cudaMalloc(&c->d_fill_zoff, (size_t)nchains * 2 * (m.lz + 1) * sizeof(int)));
        c->fill_n.assign((size_t)nchains * 2, 0);
        c->fill_zoff.assign((size_t)nchains * 2 * (m.lz + 1), 0);
        if (!weib)   // odd edge: only the padding column is outside
            for (int i = 0; i < nchains; ++i) std::fill_n(&c->mask[(size_t)i * box], box, (uint8_t)1);
        for (int i = 0; i < nchains; ++i) {
            int rc2 = upload_mask_chain(*c, i);
            if (rc2) {
                destroy_ctx(c);
                return rc2;
            }
        }
    }
    // (beta, H) float4 per chain, then H in FP64 (3 per chain): one block, one upload
    NMMC_TRY(cudaMalloc(&c->d_bh, (sizeof(float4) + 3 * sizeof(double)) * nchains));
    c->d_Hd = reinterpret_cast<double*>(c->d_bh + nchains);
    NMMC_TRY(cudaMalloc(&c->d_sweep, sizeof(unsigned long long) * nchains));
    NMMC_TRY(cudaMemset(c->d_sweep, 0, sizeof(unsigned long long) * nchains));
    NMMC_TRY(cudaMalloc(&c->d_all, sizeof(int) * nchains));
    NMMC_TRY(cudaMalloc(&c->d_list, sizeof(int) * nchains));
    NMMC_TRY(cudaMalloc(&c->d_active, nchains));
    NMMC_TRY(cudaMalloc(&c->d_pos, sizeof(int) * nchains));
    NMMC_TRY(cudaMalloc(&c->d_obs, sizeof(double) * NMMC_OBS_N * nchains));
    NMMC_TRY(cudaMalloc(&c->d_q, sizeof(double) * c->nslices * nchains));
    NMMC_TRY(cudaMalloc(&c->d_acc, sizeof(double) * NMMC_ACC_N * nchains));
    NMMC_TRY(cudaMemset(c->d_acc, 0, sizeof(double) * NMMC_ACC_N * nchains));
    NMMC_TRY(cudaMalloc(&c->d_flag, sizeof(int)));
    NMMC_TRY(cudaMemset(c->d_flag, 0, sizeof(int)));
    NMMC_TRY(cudaHostAlloc(&c->h_bh, (sizeof(float4) + 3 * sizeof(double)) * nchains, cudaHostAllocDefault));
    c->h_hd = reinterpret_cast<double*>(c->h_bh + nchains);
    NMMC_TRY(cudaHostAlloc(&c->h_list, sizeof(int) * nchains, cudaHostAllocDefault));
    NMMC_TRY(cudaEventCreateWithFlags(&c->ev_params, cudaEventDisableTiming));
    NMMC_TRY(cudaEventCreateWithFlags(&c->ev_list, cudaEventDisableTiming));
    NMMC_TRY(cudaMalloc(&c->d_rm, sizeof(ReplayModel)));
    NMMC_TRY(cudaMemcpy(c->d_rm, &c->rm, sizeof(ReplayModel), cudaMemcpyHostToDevice));
    if (!goff.empty()) {
        const size_t n = goff.size();
        NMMC_TRY(cudaMalloc(&c->d_goff, n * sizeof(int4)));
        NMMC_TRY(cudaMalloc(&c->d_gjs, n * sizeof(float4)));
        NMMC_TRY(cudaMalloc(&c->d_gje, n * sizeof(float4)));
        NMMC_TRY(cudaMalloc(&c->d_gjed, n * 4 * sizeof(double)));
        NMMC_TRY(cudaMemcpy(c->d_goff, goff.data(), n * sizeof(int4), cudaMemcpyHostToDevice));
        NMMC_TRY(cudaMemcpy(c->d_gje, c->h_gje.data(), n * sizeof(float4), cudaMemcpyHostToDevice));
        NMMC_TRY(cudaMemcpy(c->d_gjed, gjed.data(), n * 4 * sizeof(double), cudaMemcpyHostToDevice));
        c->m.g_off = c->d_goff;
        c->m.g_js = c->d_gjs;
        c->m.g_je = c->d_gje;
        c->m.g_jed = c->d_gjed;
    }
    {
        std::vector<int> all(nchains);
        for (int i = 0; i < nchains; ++i) all[i] = i;
        NMMC_TRY(cudaMemcpy(c->d_all, all.data(), sizeof(int) * nchains, cudaMemcpyHostToDevice));
    }
#undef NMMC_TRY
    rc = launch_init_spins(*c);
    if (!rc) rc = upload_params(*c);
    if (!rc) rc = upload_general(*c);
    if (!rc) rc = cuda_check(cudaStreamSynchronize(c->stream), "nmmc_create");
    if (rc) {
        destroy_ctx(c);
        return rc;
    }
    *out = c;
    return NMMC_OK;
}

void nmmc_destroy(nmmc_ctx* ctx) {
    if (ctx) cudaStreamSynchronize(ctx->stream);
    destroy_ctx(ctx);
}

int nmmc_get_info(const nmmc_ctx* c, nmmc_info* info) {
    if (!c || !info) return set_error(NMMC_ERR_ARG, "null argument");
    info->dim = c->dim;
    info->edge = c->edge;
    info->is_ising = c->ising;
    info->is_perio = c->periodic;
    info->nchains = c->nchains;
    info->nslices = c->nslices;
    info->box_sites = c->box_sites;
    info->shape_code = c->shape;
    return NMMC_OK;
}

int nmmc_site_counts(const nmmc_ctx* c, int chain, int* num, int* snum, int* s4num) {
    if (!c || chain < 0 || chain >= c->nchains) return set_error(NMMC_ERR_ARG, "bad chain");
    if (num) *num = c->num[chain];
    if (snum) *snum = c->snum[chain];
    if (s4num) *s4num = c->s4num[chain];
    return NMMC_OK;
}

int nmmc_set_point(nmmc_ctx* c, int chain, double T, double H) {
    if (!c || chain < 0 || chain >= c->nchains) return set_error(NMMC_ERR_ARG, "bad chain");
    if (!(T > 0)) return set_error(NMMC_ERR_TEMP, "Invalid temperature");
    c->T[chain] = T;
    c->H[chain] = H;
    c->params_dirty = true;
    return NMMC_OK;
}

int nmmc_get_point(const nmmc_ctx* c, int chain, double* T, double* H) {
    if (!c || chain < 0 || chain >= c->nchains) return set_error(NMMC_ERR_ARG, "bad chain");
    if (T) *T = c->T[chain];
    if (H) *H = c->H[chain];
    return NMMC_OK;
}

int nmmc_set_points(nmmc_ctx* c, const int* chains, const double* T, const double* H, int n) {
    if (!c || !chains || !T || !H) return set_error(NMMC_ERR_ARG, "null argument");
    for (int i = 0; i < n; ++i)
        if (!(T[i] > 0)) return set_error(NMMC_ERR_TEMP, "Invalid temperature");
    for (int i = 0; i < n; ++i) {
        int rc = nmmc_set_point(c, chains[i], T[i], H[i]);
        if (rc) return rc;
    }
    return NMMC_OK;
}

int nmmc_change_v1(nmmc_ctx* c, int chain, int protocol, double v1) {
    if (!c || chain < 0 || chain >= c->nchains) return set_error(NMMC_ERR_ARG, "bad chain");
    switch (protocol) {   // Old/lib/state.cpp:298-311
        case 1: case 3: return nmmc_set_point(c, chain, c->T[chain], v1);
        case 2: case 4: return nmmc_set_point(c, chain, v1, c->H[chain]);
        default: return NMMC_OK;
    }
}

int nmmc_change_v2(nmmc_ctx* c, int chain, int protocol, double v2) {
    if (!c || chain < 0 || chain >= c->nchains) return set_error(NMMC_ERR_ARG, "bad chain");
    switch (protocol) {   // Old/lib/state.cpp:313-326
        case 1: case 3: return nmmc_set_point(c, chain, v2, c->H[chain]);
        case 2: case 4: return nmmc_set_point(c, chain, c->T[chain], v2);
        default: return NMMC_OK;
    }
}

int nmmc_fork(nmmc_ctx* c, int src, int dst) {
    if (!c || src < 0 || dst < 0 || src >= c->nchains || dst >= c->nchains)
        return set_error(NMMC_ERR_ARG, "bad chain");
    if (src == dst) return NMMC_OK;
    const size_t bytes = chain_elems(*c) * elem_bytes(*c);
    NMMC_CUDA(cudaMemcpyAsync((char*)c->d_spins + dst * bytes, (char*)c->d_spins + src * bytes, bytes,
                              cudaMemcpyDeviceToDevice, c->stream));
    if (c->masked && memcmp(&c->mask[(size_t)src * c->box_sites], &c->mask[(size_t)dst * c->box_sites],
                            (size_t)c->box_sites) != 0) {
        // the copy takes the particle with it: shape, counts and tables follow the source
        std::copy_n(&c->mask[(size_t)src * c->box_sites], c->box_sites, &c->mask[(size_t)dst * c->box_sites]);
        c->num[dst] = c->num[src];
        c->snum[dst] = c->snum[src];
        c->s4num[dst] = c->s4num[src];
        c->size[dst] = c->size[src];
        NMMC_CUDA(cudaStreamSynchronize(c->stream));
        int rc = upload_mask_chain(*c, dst);
        if (rc) return rc;
        resident_free(*c);
    }
    c->T[dst] = c->T[src];
    c->H[dst] = c->H[src];
    c->params_dirty = true;
    return NMMC_OK;
}

int nmmc_sweep(nmmc_ctx* c, const int* chains, int n, int nsweeps) {
    if (!c) return set_error(NMMC_ERR_ARG, "null context");
    chains = all_if_identity(*c, chains, n);
    if (nsweeps < 0) return set_error(NMMC_ERR_ARG, "negative sweep count");
    const int* d = nullptr;
    int rc = set_list(*c, chains, n, &d);
    if (rc) return rc;
    if (!chains) n = c->nchains;
    return sweep_impl(*c, d, chains, n, nsweeps, true);
}

int nmmc_measure(nmmc_ctx* c, const int* chains, int n, double* obs, double* q, int accumulate) {
    if (!c || (!obs && q)) return set_error(NMMC_ERR_ARG, "null argument");
    chains = all_if_identity(*c, chains, n);
    const int* d = nullptr;
    int rc = set_list(*c, chains, n, &d);
    if (rc) return rc;
    if (!chains) n = c->nchains;
    if (n == 0) return NMMC_OK;   // an empty list measures nothing
    if ((rc = upload_params(*c))) return rc;
    if ((rc = launch_measure(*c, d, n, accumulate))) return rc;
    if (accumulate && (rc = launch_add_av(*c))) return rc;
    if (!obs) return NMMC_OK;   // results stay on the device (accumulators), no synchronisation
    NMMC_CUDA(cudaMemcpyAsync(obs, c->d_obs, sizeof(double) * NMMC_OBS_N * n, cudaMemcpyDeviceToHost, c->stream));
    if (q)
        NMMC_CUDA(cudaMemcpyAsync(q, c->d_q, sizeof(double) * c->nslices * n, cudaMemcpyDeviceToHost, c->stream));
    NMMC_CUDA(cudaStreamSynchronize(c->stream));
    return NMMC_OK;
}

int nmmc_sweep_measure(nmmc_ctx* c, const int* chains, int n, int nsweeps, double* obs, double* q, int accumulate) {
    if (!c || (!obs && q)) return set_error(NMMC_ERR_ARG, "null argument");
    chains = all_if_identity(*c, chains, n);
    if (nsweeps < 0) return set_error(NMMC_ERR_ARG, "negative sweep count");
    const int* d = nullptr;
    int rc = set_list(*c, chains, n, &d);
    if (rc) return rc;
    if (!chains) n = c->nchains;
    if (n == 0) return NMMC_OK;   // an empty list sweeps and measures nothing
    if ((rc = measure_prepare(*c, n))) return rc;
    if ((rc = sweep_measure_impl(*c, d, chains, n, nsweeps, accumulate, true))) return rc;
    if (!obs) return NMMC_OK;   // results stay on the device (accumulators), no synchronisation
    NMMC_CUDA(cudaMemcpyAsync(obs, c->d_obs, sizeof(double) * NMMC_OBS_N * n, cudaMemcpyDeviceToHost, c->stream));
    if (q)
        NMMC_CUDA(cudaMemcpyAsync(q, c->d_q, sizeof(double) * c->nslices * n, cudaMemcpyDeviceToHost, c->stream));
    NMMC_CUDA(cudaStreamSynchronize(c->stream));
    return NMMC_OK;
}

int nmmc_sample(nmmc_ctx* c, const int* chains, int n, int nsweeps, int nsamples, double* obs, double* q) {
    if (!c || !obs || nsamples < 0 || nsweeps < 0) return set_error(NMMC_ERR_ARG, "bad argument");
    if (chains) {
        if (int rc = check_list(*c, chains, n)) return rc;
    }
    std::vector<int> list;
    if (chains) list.assign(chains, chains + n);
    else {
        n = c->nchains;
        for (int i = 0; i < n; ++i) list.push_back(i);
    }
    if (nsamples == 0 || n == 0) return NMMC_OK;
    int rc = upload_params(*c);
    if (rc) return rc;
    if (c->sweep_path != 1) {
        if ((rc = resident_prepare(*c))) return rc;
    }
    // the HBM path's compact tables: no allocation or table upload inside the capture
    if (!(c->sweep_path != 1 && resident_chosen(*c))) {
        if ((rc = compact_prepare(*c))) return rc;
        wave_ready(*c);   // the wavefront sweeps' second array (when enabled), not inside the capture
    }
    if ((rc = measure_prepare(*c, n))) return rc;
    // history buffers on the device, one D2H at the end
    DeviceScratch ds;
    double *d_hist = nullptr, *d_qhist = nullptr;
    int* d_l = nullptr;
    NMMC_CUDA(ds.alloc(&d_hist, sizeof(double) * NMMC_OBS_N * n * (size_t)nsamples));
    if (q) NMMC_CUDA(ds.alloc(&d_qhist, sizeof(double) * c->nslices * n * (size_t)nsamples));
    NMMC_CUDA(ds.alloc(&d_l, sizeof(int) * n));
    NMMC_CUDA(cudaMemcpy(d_l, list.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    // one graph: nsweeps sweeps + measure (accumulating), as nmmc_sweep_measure
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    NMMC_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    const bool all = all_if_identity(*c, list.data(), n) == nullptr;   // every chain, in order
    rc = sweep_measure_impl(*c, all ? c->d_all : d_l, all ? nullptr : list.data(), n, nsweeps, 1, false);
    cudaError_t ce = cudaStreamEndCapture(c->stream, &g);
    if (rc || ce != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return rc ? rc : cuda_check(ce, "cudaStreamEndCapture");
    }
    ce = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) return cuda_check(ce, "cudaGraphInstantiate");
    const size_t ob = sizeof(double) * NMMC_OBS_N * n, qb = sizeof(double) * c->nslices * n;
    for (int s = 0; s < nsamples && !rc; ++s) {
        rc = cuda_check(cudaGraphLaunch(ge, c->stream), "cudaGraphLaunch");
        if (!rc) rc = cuda_check(cudaMemcpyAsync((char*)d_hist + ob * s, c->d_obs, ob, cudaMemcpyDeviceToDevice, c->stream), "obs copy");
        if (!rc && q) rc = cuda_check(cudaMemcpyAsync((char*)d_qhist + qb * s, c->d_q, qb, cudaMemcpyDeviceToDevice, c->stream), "q copy");
    }
    if (!rc) rc = cuda_check(cudaMemcpyAsync(obs, d_hist, ob * nsamples, cudaMemcpyDeviceToHost, c->stream), "obs D2H");
    if (!rc && q) rc = cuda_check(cudaMemcpyAsync(q, d_qhist, qb * nsamples, cudaMemcpyDeviceToHost, c->stream), "q D2H");
    cudaError_t se = cudaStreamSynchronize(c->stream);
    if (!rc) rc = cuda_check(se, "nmmc_sample");
    cudaGraphExecDestroy(ge);
    return rc;
}

int nmmc_get_accumulators(nmmc_ctx* c, const int* chains, int n, double* out) {
    if (!c || !out) return set_error(NMMC_ERR_ARG, "null argument");
    std::vector<double> all((size_t)NMMC_ACC_N * c->nchains);
    NMMC_CUDA(cudaStreamSynchronize(c->stream));
    NMMC_CUDA(cudaMemcpy(all.data(), c->d_acc, sizeof(double) * all.size(), cudaMemcpyDeviceToHost));
    if (!chains) n = c->nchains;
    for (int i = 0; i < n; ++i) {
        int ch = chains ? chains[i] : i;
        if (ch < 0 || ch >= c->nchains) return set_error(NMMC_ERR_ARG, "chain index out of range");
        std::copy_n(&all[(size_t)ch * NMMC_ACC_N], NMMC_ACC_N, out + (size_t)i * NMMC_ACC_N);
    }
    return NMMC_OK;
}

int nmmc_reset_accumulators(nmmc_ctx* c) {
    if (!c) return set_error(NMMC_ERR_ARG, "null context");
    NMMC_CUDA(cudaMemsetAsync(c->d_acc, 0, sizeof(double) * NMMC_ACC_N * c->nchains, c->stream));
    return NMMC_OK;
}

int nmmc_get_spins(nmmc_ctx* c, int chain, double* xyz, size_t n_sites) {
    if (!c || !xyz || chain < 0 || chain >= c->nchains) return set_error(NMMC_ERR_ARG, "bad argument");
    if (n_sites != (size_t)c->box_sites) return set_error(NMMC_ERR_ARG, "expected %lld sites", c->box_sites);
    const size_t bytes = chain_elems(*c) * elem_bytes(*c);
    std::vector<char> buf(bytes);
    NMMC_CUDA(cudaStreamSynchronize(c->stream));
    NMMC_CUDA(cudaMemcpy(buf.data(), (char*)c->d_spins + chain * bytes, bytes, cudaMemcpyDeviceToHost));
    planes_to_box(*c, buf.data(), xyz);
    return NMMC_OK;
}

int nmmc_set_spins(nmmc_ctx* c, int chain, const double* xyz, size_t n_sites) {
    if (!c || !xyz || chain < 0 || chain >= c->nchains) return set_error(NMMC_ERR_ARG, "bad argument");
    if (n_sites != (size_t)c->box_sites) return set_error(NMMC_ERR_ARG, "expected %lld sites", c->box_sites);
    const size_t bytes = chain_elems(*c) * elem_bytes(*c);
    std::vector<char> buf(bytes, 0);
    box_to_planes(*c, xyz, c->masked ? &c->mask[(size_t)chain * c->box_sites] : nullptr, buf.data());
    NMMC_CUDA(cudaStreamSynchronize(c->stream));
    NMMC_CUDA(cudaMemcpy((char*)c->d_spins + chain * bytes, buf.data(), bytes, cudaMemcpyHostToDevice));
    return NMMC_OK;
}

int nmmc_set_av_chains(nmmc_ctx* c, const int* chains, int n) {
    if (!c || n < 0 || n > c->nchains || (n && !chains)) return set_error(NMMC_ERR_ARG, "bad argument");
    for (int i = 0; i < n; ++i) {
        if (chains[i] < 0 || chains[i] >= c->nchains) return set_error(NMMC_ERR_ARG, "chain index out of range");
        for (int k = 0; k < i; ++k)
            if (chains[k] == chains[i]) return set_error(NMMC_ERR_ARG, "chain %d listed twice", chains[i]);
    }
    NMMC_CUDA(cudaStreamSynchronize(c->stream));
    c->av_chains.assign(chains, chains + n);
    if (!n) return NMMC_OK;
    if ((size_t)n > c->av_cap) {
        cudaFree(c->d_av);
        cudaFree(c->d_av_list);
        c->d_av = nullptr;
        c->d_av_list = nullptr;
        c->av_cap = 0;
        NMMC_CUDA(cudaMalloc(&c->d_av, sizeof(double) * 3 * (size_t)c->box_sites * n));
        NMMC_CUDA(cudaMalloc(&c->d_av_list, sizeof(int) * n));
        c->av_cap = (size_t)n;
    }
    NMMC_CUDA(cudaMemcpy(c->d_av_list, chains, sizeof(int) * n, cudaMemcpyHostToDevice));
    NMMC_CUDA(cudaMemset(c->d_av, 0, sizeof(double) * 3 * (size_t)c->box_sites * n));
    return NMMC_OK;
}

int nmmc_get_av(nmmc_ctx* c, int chain, double* xyz, size_t n_sites) {
    if (!c || !xyz) return set_error(NMMC_ERR_ARG, "null argument");
    if (n_sites != (size_t)c->box_sites) return set_error(NMMC_ERR_ARG, "expected %lld sites", c->box_sites);
    size_t slot = 0;
    while (slot < c->av_chains.size() && c->av_chains[slot] != chain) ++slot;
    if (slot == c->av_chains.size()) return set_error(NMMC_ERR_ARG, "chain %d is not summed (nmmc_set_av_chains)", chain);
    NMMC_CUDA(cudaStreamSynchronize(c->stream));
    NMMC_CUDA(cudaMemcpy(xyz, c->d_av + slot * 3 * (size_t)c->box_sites, sizeof(double) * 3 * (size_t)c->box_sites,
                         cudaMemcpyDeviceToHost));
    return NMMC_OK;
}

int nmmc_get_mask(nmmc_ctx* c, int chain, uint8_t* mask, size_t n_sites) {
    if (!c || !mask || chain < 0 || chain >= c->nchains) return set_error(NMMC_ERR_ARG, "bad argument");
    if (n_sites != (size_t)c->box_sites) return set_error(NMMC_ERR_ARG, "expected %lld sites", c->box_sites);
    std::copy_n(&c->mask[(size_t)chain * c->box_sites], c->box_sites, mask);
    return NMMC_OK;
}

int nmmc_delta_e(nmmc_ctx* c, int chain, const int32_t* sites, const double* trial, int n, double* dE) {
    if (!c || !sites || !trial || !dE || n < 0 || chain < 0 || chain >= c->nchains)
        return set_error(NMMC_ERR_ARG, "bad argument");
    if (n == 0) return NMMC_OK;
    for (int i = 0; i < n; ++i) {
        if (sites[i] < 0 || sites[i] >= c->box_sites) return set_error(NMMC_ERR_ARG, "site %d out of range", sites[i]);
        if (!c->mask[(size_t)chain * c->box_sites + sites[i]]) return set_error(NMMC_ERR_ARG, "site %d is outside the particle", sites[i]);
    }
    int rc = upload_params(*c);
    if (rc) return rc;
    std::vector<float> tf(3 * (size_t)n);
    for (size_t i = 0; i < tf.size(); ++i) tf[i] = (float)trial[i];
    DeviceScratch ds;
    int32_t* d_sites = nullptr;
    float* d_trial = nullptr;
    double* d_out = nullptr;
    NMMC_CUDA(ds.alloc(&d_sites, sizeof(int32_t) * n));
    NMMC_CUDA(ds.alloc(&d_trial, sizeof(float) * 3 * n));
    NMMC_CUDA(ds.alloc(&d_out, sizeof(double) * n));
    NMMC_CUDA(cudaMemcpyAsync(d_sites, sites, sizeof(int32_t) * n, cudaMemcpyHostToDevice, c->stream));
    NMMC_CUDA(cudaMemcpyAsync(d_trial, tf.data(), sizeof(float) * 3 * n, cudaMemcpyHostToDevice, c->stream));
    rc = c->m.general ? launch_delta_e_general(*c, chain, d_sites, d_trial, n, d_out)
                      : launch_delta_e(*c, chain, d_sites, d_trial, n, d_out);
    if (!rc) rc = cuda_check(cudaMemcpyAsync(dE, d_out, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream), "dE D2H");
    // the scratch is freed on return: the stream is drained first whatever happened above
    const cudaError_t se = cudaStreamSynchronize(c->stream);
    if (!rc) rc = cuda_check(se, "nmmc_delta_e");
    return rc;
}

int nmmc_debug_replay(nmmc_ctx* c, int chain, const nmmc_event* ev, size_t n, uint8_t* accepted,
                      int64_t* first_mismatch, double* final_xyz) {
    if (!c || (!ev && n) || chain < 0 || chain >= c->nchains) return set_error(NMMC_ERR_ARG, "bad argument");
    for (size_t i = 0; i < n; ++i) {
        int s = ev[i].site_box;
        if (s < 0 || s >= c->box_sites) return set_error(NMMC_ERR_ARG, "event %zu: site %d out of range", i, s);
        if (!c->mask[(size_t)chain * c->box_sites + s]) return set_error(NMMC_ERR_ARG, "event %zu: site %d outside the particle", i, s);
        if (ev[i].u <= 0 && ev[i].accepted == 0) return set_error(NMMC_ERR_ARG, "event %zu: rejection without a uniform", i);
    }
    c->rm.dmi_sign = c->dmi_sign;
    NMMC_CUDA(cudaMemcpyAsync(c->d_rm, &c->rm, sizeof(ReplayModel), cudaMemcpyHostToDevice, c->stream));
    if (!c->d_replay) NMMC_CUDA(cudaMalloc(&c->d_replay, sizeof(double) * 3 * (size_t)c->box_sites));
    DeviceScratch ds;
    nmmc_event* d_ev = nullptr;
    uint8_t* d_acc = nullptr;
    long long* d_first = nullptr;
    NMMC_CUDA(ds.alloc(&d_ev, sizeof(nmmc_event) * std::max<size_t>(1, n)));
    NMMC_CUDA(ds.alloc(&d_acc, std::max<size_t>(1, n)));
    NMMC_CUDA(ds.alloc(&d_first, sizeof(long long)));
    int rc = NMMC_OK;
    if (n) rc = cuda_check(cudaMemcpyAsync(d_ev, ev, sizeof(nmmc_event) * n, cudaMemcpyHostToDevice, c->stream), "events H2D");
    if (!rc) rc = launch_replay(*c, chain, d_ev, n, d_acc, d_first);
    long long first = -1;
    int flag = 0;
    if (!rc && accepted && n) rc = cuda_check(cudaMemcpyAsync(accepted, d_acc, n, cudaMemcpyDeviceToHost, c->stream), "acc D2H");
    if (!rc) rc = cuda_check(cudaMemcpyAsync(&first, d_first, sizeof(long long), cudaMemcpyDeviceToHost, c->stream), "first D2H");
    if (!rc) rc = cuda_check(cudaMemcpyAsync(&flag, c->d_flag, sizeof(int), cudaMemcpyDeviceToHost, c->stream), "flag D2H");
    if (!rc && final_xyz)
        rc = cuda_check(cudaMemcpyAsync(final_xyz, c->d_replay, sizeof(double) * 3 * c->box_sites, cudaMemcpyDeviceToHost, c->stream), "final D2H");
    const cudaError_t se = cudaStreamSynchronize(c->stream);   // drained before the scratch is freed
    if (!rc) rc = cuda_check(se, "nmmc_debug_replay");
    if (rc) return rc;
    if (flag) {
        cudaMemset(c->d_flag, 0, sizeof(int));
        return set_error(NMMC_ERR_ARG, "replay stopped at an invalid site (code %d)", flag);
    }
    if (first_mismatch) *first_mismatch = first;
    return NMMC_OK;
}

int nmmc_set_option(nmmc_ctx* c, int key, int64_t v) {
    if (!c) return set_error(NMMC_ERR_ARG, "null context");
    switch (key) {
        case NMMC_OPT_SWEEP_PATH:
            if (v < 0 || v > 2) return set_error(NMMC_ERR_ARG, "sweep path must be 0, 1 or 2");
            c->sweep_path = (int)v;
            break;
        case NMMC_OPT_DMI_SIGN:
            if (v != 0 && v != 1) return set_error(NMMC_ERR_ARG, "dmi sign must be 0 or 1");
            c->dmi_sign = (int)v;
            for (int k = 0; k < 6; ++k)
                for (int a = 0; a < 3; ++a) c->m.Ds[k][a] = v ? -c->m.De[k][a] : c->m.De[k][a];
            classify_dmi(c->m);
            if (int rc = upload_general(*c)) return rc;
            break;
        case NMMC_OPT_MEASURE_FP64: c->measure_fp64 = v ? 1 : 0; break;
        case NMMC_OPT_HALF_KERNEL:
            if (v < 0 || v > 8) return set_error(NMMC_ERR_ARG, "half kernel must be 0..8");
            c->half_kernel = (int)v;
            break;
        case NMMC_OPT_WAIT_LIMIT:
            if (v < 0 || v > 0xffffffffLL) return set_error(NMMC_ERR_ARG, "wait limit must be 0 .. 2^32-1");
            c->wait_limit = (unsigned)v;
            break;
        case NMMC_OPT_RING_ZSEG:
            if (v < 0 || v > 4096) return set_error(NMMC_ERR_ARG, "ring z-segment must be 0 .. 4096");
            c->ring_zseg = (int)v;
            break;
        case NMMC_OPT_L2_PREFETCH:
            if (v < 0 || v > 64) return set_error(NMMC_ERR_ARG, "L2 prefetch distance must be 0 .. 64");
            c->l2_prefetch = (int)v;
            break;
        case NMMC_OPT_WAVE:
            if (v != 0 && v != 1) return set_error(NMMC_ERR_ARG, "wave must be 0 or 1");
            c->wave = (int)v;
            break;
        case NMMC_OPT_PERIODIC_Q: c->periodic_q = v ? 1 : 0; c->m.periodic_q = c->periodic_q; break;
        case NMMC_OPT_TIMING: c->timing = v ? 1 : 0; break;
        case NMMC_OPT_RESIDENT_THREADS:
            if (v != 0 && (v < 32 || v > 1024 || v % 32)) return set_error(NMMC_ERR_ARG, "threads must be a multiple of 32 up to 1024");
            c->res_threads = (int)v;
            resident_free(*c);
            break;
        case NMMC_OPT_MEASURE_SITES:
            if (v != 2 && v != 4) return set_error(NMMC_ERR_ARG, "measurement sites per item must be 2 or 4");
            c->measure_sites = (int)v;
            break;
        case NMMC_OPT_RESIDENT_BINS:
            if (v < 0) return set_error(NMMC_ERR_ARG, "bins must be >= 0");
            c->res_bins = (int)v;
            resident_free(*c);
            break;
        case NMMC_OPT_MASKED_COMPACT:
            if (v != 0 && v != 1) return set_error(NMMC_ERR_ARG, "masked compact must be 0 or 1");
            c->masked_compact = (int)v;
            break;
        case NMMC_OPT_RESIDENT_PREDRAW:
            if (v < 0 || v > 2) return set_error(NMMC_ERR_ARG, "predraw must be 0, 1 or 2");
            c->res_predraw = (int)v;
            resident_free(*c);
            break;
        case NMMC_OPT_CHARGE_PASS:
            if (v != 0 && v != 1) return set_error(NMMC_ERR_ARG, "charge pass must be 0 or 1");
            c->charge_pass = (int)v;
            break;
        case NMMC_OPT_RESIDENT_STENCIL:
            if (v < 0 || v > 2) return set_error(NMMC_ERR_ARG, "stencil must be 0, 1 or 2");
            c->res_stencil = (int)v;
            resident_free(*c);
            break;
        default: return set_error(NMMC_ERR_ARG, "unknown option %d", key);
    }
    return NMMC_OK;
}

int nmmc_get_option(const nmmc_ctx* c, int key, int64_t* v) {
    if (!c || !v) return set_error(NMMC_ERR_ARG, "null argument");
    switch (key) {
        case NMMC_OPT_SWEEP_PATH: *v = c->sweep_path; break;
        case NMMC_OPT_DMI_SIGN: *v = c->dmi_sign; break;
        case NMMC_OPT_MEASURE_FP64: *v = c->measure_fp64; break;
        case NMMC_OPT_HALF_KERNEL: *v = c->half_kernel; break;
        case NMMC_OPT_PERIODIC_Q: *v = c->periodic_q; break;
        case NMMC_OPT_TIMING: *v = c->timing; break;
        case NMMC_OPT_RESIDENT_THREADS: *v = c->res.built ? c->res.threads : c->res_threads; break;
        case NMMC_OPT_COLOURS: *v = c->m.col_q; break;
        case NMMC_OPT_MEASURE_SITES: *v = c->measure_sites; break;
        case NMMC_OPT_RESIDENT_BINS: *v = c->res.built ? c->res.nbins : c->res_bins; break;
        case NMMC_OPT_RESIDENT_PREDRAW: *v = c->res.built ? (c->res.predraw ? 2 : 1) : c->res_predraw; break;
        case NMMC_OPT_MASKED_COMPACT: *v = c->masked_compact; break;
        case NMMC_OPT_WAIT_LIMIT: *v = c->wait_limit; break;
        case NMMC_OPT_RING_ZSEG: *v = c->ring_zseg; break;
        case NMMC_OPT_L2_PREFETCH: *v = c->l2_prefetch; break;
        case NMMC_OPT_WAVE: *v = c->wave; break;
        case NMMC_OPT_CHARGE_PASS: *v = c->charge_pass; break;
        case NMMC_OPT_RESIDENT_STENCIL: *v = c->res.built ? (c->res.stencil ? 2 : 1) : c->res_stencil; break;
        default: return set_error(NMMC_ERR_ARG, "unknown option %d", key);
    }
    return NMMC_OK;
}

int nmmc_get_timing(nmmc_ctx* c, double* ms, long long* launches, long long* updates) {
    if (!c) return set_error(NMMC_ERR_ARG, "null context");
    int rc = resolve_timing(*c);
    if (rc) return rc;
    if (ms) *ms = c->t_ms;
    if (launches) *launches = c->t_launches;
    if (updates) *updates = c->t_updates;
    c->t_ms = 0;
    c->t_launches = 0;
    c->t_updates = 0;
    return NMMC_OK;
}

int nmmc_timer_mark(nmmc_ctx* c, int slot) {
    if (!c || slot < 0 || slot >= 8) return set_error(NMMC_ERR_ARG, "bad timer slot");
    if (!c->marks[slot]) NMMC_CUDA(cudaEventCreate(&c->marks[slot]));
    NMMC_CUDA(cudaEventRecord(c->marks[slot], c->stream));
    return NMMC_OK;
}

int nmmc_timer_elapsed(nmmc_ctx* c, int a, int b, double* ms) {
    if (!c || !ms || a < 0 || b < 0 || a >= 8 || b >= 8 || !c->marks[a] || !c->marks[b])
        return set_error(NMMC_ERR_ARG, "bad timer slot");
    NMMC_CUDA(cudaEventSynchronize(c->marks[b]));
    float f = 0;
    NMMC_CUDA(cudaEventElapsedTime(&f, c->marks[a], c->marks[b]));
    *ms = f;
    return NMMC_OK;
}

int nmmc_host_alloc(size_t bytes, void** out) {
    if (!out || !bytes) return set_error(NMMC_ERR_ARG, "bad argument");
    *out = nullptr;
    cudaError_t e = cudaHostAlloc(out, bytes, cudaHostAllocDefault);
    if (e != cudaSuccess) return cuda_check(e, "cudaHostAlloc");
    return NMMC_OK;
}

int nmmc_host_free(void* p) {
    if (!p) return NMMC_OK;
    return cuda_check(cudaFreeHost(p), "cudaFreeHost");
}

void* nmmc_stream(nmmc_ctx* c) { return c ? (void*)c->stream : nullptr; }

int nmmc_synchronize(nmmc_ctx* c) {
    if (!c) return set_error(NMMC_ERR_ARG, "null context");
    NMMC_CUDA(cudaStreamSynchronize(c->stream));
    int flag = 0;
    NMMC_CUDA(cudaMemcpy(&flag, c->d_flag, sizeof(int), cudaMemcpyDeviceToHost));
    if (flag == 3) {
        cudaMemset(c->d_flag, 0, sizeof(int));
        return set_error(NMMC_ERR_TIMEOUT, "a pipelined sweep gave up waiting for its copies");
    }
    return NMMC_OK;
}

}  // extern "C"
