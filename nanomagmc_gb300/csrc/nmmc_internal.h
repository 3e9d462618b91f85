// Internal definitions shared by the CUDA translation units of libnmmc.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <string>
#include <vector>

#include "../../include/nmmc.h"
#include "nmmc_hostlib.h"
#include "philox.h"

namespace nmmc {

// Direction order of the stencil: +x, -x, +y, -y, +z, -z.
constexpr int kMaxDir = 6;

// Lattice, couplings and RNG key, passed by value to every kernel.
//
// Spin storage ("split-colour SoA"): for chain c, colour p = (x+y+z)&1 and component k,
// plane(c,p,k) = spins + ((c*2 + p)*ncomp + k) * nhalf_pad, where ncomp = 3 (Heisenberg,
// FP32) or 1 (Ising, int8). Inside a plane a site sits at ((z*ly + y)*hx + (x>>1)).
// Rows are lx = edge rounded up to even, so every row holds hx = lx/2 sites of each colour;
// padding columns (x >= edge) are outside the particle. Sites outside the particle hold 0.
struct DevModel {
    int dim, edge, lx, ly, lz, hx;
    int nhalf, nhalf_pad;
    int periodic, ising, masked;
    int periodic_q;
    int has_dmi;
    int dmi_kind;             // kDmi* (nmmc_kernels.cuh): structure of Ds used by the sweeps
    int ndir;                 // 4 in 2-D, 6 in 3-D
    float J[kMaxDir];         // exchange per direction (sum of the records on that offset)
    float Ds[kMaxDir][3];     // DMI vector of the sweep: local field += s_k x Ds_k
    float De[kMaxDir][3];     // DMI vector of the energy: e_i += s_i . (De_k x s_k)
    double Jd[kMaxDir];       // FP64 copies for the FP64 measurement mode
    double Ded[kMaxDir][3];
    uint32_t key0, key1;
    uint32_t rk0[10], rk1[10];   // Philox round keys (key + r * Weyl constants)
    int qpr_shift, ly_shift;     // log2 of (hx/4) and of ly when they are powers of two, else -1
    // General interaction table (any offsets; J, Ds, De above are then zero): the coupling
    // records in file order, swept colour class by colour class (nmmc_general.cu).
    int general;                 // 1: general table
    int ngen;                    // coupling records
    int col_kind, col_q, col_p, col_b, col_c;   // colouring (Colouring in nmmc_hostlib.h)
    const int4* g_off;           // per record: offset x, y, z (0 beyond dim; wrapped into [0, edge)
                                 // on periodic lattices), 1 if the record lands on the site itself
    const float4* g_js;          // per record: J, Ds (sweep convention, follows the DMI sign)
    const float4* g_je;          // per record: J, De (energy convention)
    const double* g_jed;         // per record: J, De in FP64 (4 doubles)
};

// The original interaction records, kept in file order for the FP64 sequential replay (held
// in device memory: with NMMC_MAX_OFFSETS records it exceeds the kernel parameter space).
struct ReplayModel {
    int n;
    int off[NMMC_MAX_OFFSETS][3];
    double J[NMMC_MAX_OFFSETS];
    double D[NMMC_MAX_OFFSETS][3];
    int useJ, useD, dmi_sign;
};

// Tables of the shared-memory resident sweep kernel (one bin = the chains one CTA owns).
struct ResidentTables {
    bool built = false;
    bool eligible = false;
    int nbins = 0, threads = 0, cap = 0;   // cap: max sites in a bin (smem sizing; the zero site)
    int total_sites = 0;
    int tables_bins = 0;          // bin count the tables below were built for
    uint32_t* d_goff = nullptr;   // per site: offset of component 0 in the spin array
    uint4* d_rec = nullptr;       // per site: neighbours, box index and slot (nmmc_resident.cu)
    int* d_bin_begin = nullptr;   // nbins+1 site offsets
    int* d_bin_nred = nullptr;    // red (colour 0) sites of each bin, stored first
    int* d_bin_chain_begin = nullptr;  // nbins+1 offsets into d_bin_chains
    int* d_bin_chains = nullptr;
    int* d_slot_red = nullptr;    // per d_bin_chains entry: bin-local first colour-0 site
    int* d_slot_black = nullptr;  // per d_bin_chains entry: bin-local first colour-1 site
    // Drawn-ahead variant (few bins): a separate kernel writes the Philox words of the next
    // sweeps of every site, so that the resident kernel's updates skip the generator.
    bool hbm_faster = false;      // the autotuner timed the HBM path faster: the automatic path takes it
    bool stencil = false;         // sweeps run on the stencil resident kernel (nmmc_stencil.cu)
    bool predraw = false;         // the shape in use launches the drawn-ahead variant
    int* d_site_chain = nullptr;  // per site: its chain
    uint4* d_draws = nullptr;     // [sweep of the launch][site] Philox words
    int draw_sweeps = 0;          // sweeps d_draws holds (longer calls are split)
};

struct TimedCall {
    cudaEvent_t a = nullptr, b = nullptr;
    long long launches = 0, updates = 0;
};

struct Ctx {
    // lattice
    DevModel m{};
    ReplayModel rm{};
    ReplayModel* d_rm = nullptr;        // device copy for the replay kernel
    Colouring col;                      // colour classes of the sweep (kind 0: checkerboard)
    std::vector<float4> h_gje;          // general records, energy convention (host copy)
    int4* d_goff = nullptr;             // general records on the device (DevModel g_*)
    float4* d_gjs = nullptr;
    float4* d_gje = nullptr;
    double* d_gjed = nullptr;
    int dim = 2, edge = 0, nchains = 0, nslices = 1;
    long long box_sites = 0;
    bool ising = false, periodic = false, masked = false;
    char shape = 's';
    double k_b = 1.0;
    uint64_t seed = 0;
    std::vector<double> T, H, size;
    std::vector<uint8_t> mask;          // nchains x box_sites (logical box), 1 = filled
    std::vector<int> num, snum, s4num;  // site counts per chain
    nmmc_interactions inter{};

    // device state
    cudaStream_t stream = nullptr;
    int device = 0;                     // CUDA device the context was created on
    int sm_count = 0;
    size_t smem_optin = 0;
    std::string gpu_name;
    void* d_spins = nullptr;            // float (Heisenberg) or int8 (Ising) planes
    size_t spins_bytes = 0;
    // second spin array of the wavefront sweeps (out of place: each sweep reads one array and
    // writes the other, an even number of them per call so that d_spins holds the result);
    // allocated at the first such sweep
    void* d_spins_alt = nullptr;
    bool wave_no_memory = false;        // the second array could not be allocated: half-sweeps only
    int wave_per_sm[8] = {};            // resident CTAs per SM of each wavefront kernel (0: not queried)
    int pf_per_sm[16] = {};             // the same for each prefetching half-sweep kernel
    size_t stencil_smem[16] = {};       // dynamic shared memory set for each stencil resident kernel
    uint8_t* d_mask = nullptr;          // split-colour mask planes (nullptr: unmasked)
    // masked lattices: per chain and colour, the compact indices of the filled sites in
    // increasing order (segment (chain * 2 + colour) of nhalf entries) and their counts, so
    // that the HBM half-sweeps launch threads for filled sites only
    uint32_t* d_fill = nullptr;
    int* d_fill_n = nullptr;
    std::vector<int> fill_n;            // host copy of the counts
    int fill_max = 0;                   // largest count (grid size)
    // per chain and colour, lz + 1 offsets into its list: the entries of z-slice z are
    // [zoff[z], zoff[z + 1]) (the measurement's blocks cover one slice each)
    int* d_fill_zoff = nullptr;
    std::vector<int> fill_zoff;
    int fill_slice_max = 0;             // most filled sites (both colours) of one slice
    // masked Heisenberg lattices on the HBM path, compact form: per chain and colour, the
    // filled sites' spins in list order (nhalf float4 x, y, z, 0) and a table per site: packed, one
    // int4 of the 2*dim neighbours' list indices in the other colour as 16-bit differences to
    // the site's own index (kNoNeighbour16: an empty site) and the box index; where a
    // difference does not fit, two int4 of absolute indices (-1: empty) and the box index.
    // Built at the first such sweep, kept in step with the masks on fork.
    float4* d_cspins = nullptr;         // [chain * 2 + colour][nhalf] (x, y, z, 0)
    int4* d_ctab = nullptr;
    bool ctab_built = false;
    bool ctab_packed = true;
    float4* d_bh = nullptr;             // per chain (beta, H0, H1, H2) in FP32
    double* d_Hd = nullptr;             // per chain H in FP64 (3 doubles) for the energy
    unsigned long long* d_sweep = nullptr;  // per chain sweep counter
    int* d_all = nullptr;               // 0..nchains-1
    int* d_list = nullptr;              // chain list of the current call
    uint8_t* d_active = nullptr;        // per chain: part of the current resident call
    int* d_pos = nullptr;               // per chain: its position in the current call's list
    bool active_all = false;            // d_active marks every chain (set by direct calls only)
    double* d_partial = nullptr;        // measure partials
    size_t partial_cap = 0;             // doubles
    double* d_mrows = nullptr;          // block rows of the fused half-sweeps (nmmc_sweep_measure, HBM path)
    size_t mrows_cap = 0;               // doubles
    double* d_obs = nullptr;            // nchains x NMMC_OBS_N
    double* d_q = nullptr;              // nchains x nslices
    double* d_acc = nullptr;            // nchains x NMMC_ACC_N
    double* d_replay = nullptr;         // FP64 working copy for the sequential replay
    int* d_flag = nullptr;              // device error word
    // pinned host staging of the per-call uploads; each is reused only after its last copy
    float4* h_bh = nullptr;             // nchains
    double* h_hd = nullptr;             // 3 x nchains
    int* h_list = nullptr;              // nchains
    cudaEvent_t ev_params = nullptr, ev_list = nullptr;
    std::vector<int> av_chains;         // chains summed by add_to_av (nmmc_set_av_chains)
    int* d_av_list = nullptr;           // the same list on the device
    double* d_av = nullptr;             // per listed chain: box_sites x 3 FP64 sums, x fastest
    size_t av_cap = 0;                  // chains d_av holds
    bool params_dirty = true;

    // options
    int sweep_path = 0, dmi_sign = 0, measure_fp64 = 0, periodic_q = 0, timing = 0;
    int res_threads = 0, res_bins = 0;
    int res_predraw = 0;   // resident drawn-ahead variant: 0 autotuned, 1 off, 2 on where it fits
    int res_stencil = 0;   // stencil resident kernel: 0 autotuned, 1 off, 2 on where the lattice fits
    int masked_compact = 0;  // masked Heisenberg HBM sweeps: 0 compact form, 1 over the box layout
    int half_kernel = 0;   // 0: widest applicable HBM kernel, 1: one site per thread
    int measure_sites = 2; // sites per thread item of the streaming measurement kernel (2 or 4)
    int charge_pass = 0;   // charge pass after fused half-sweeps: 0 sliding rows (k_charge_rows), 1 k_measure_q4 items
    int wave = 0;          // HBM path: 1 runs full sweeps as one wavefront launch where the lattice allows
    int l2_prefetch = 2;   // four-site half-sweeps: L2 prefetch distance in quarter waves of resident blocks (0: off)
    int ring_zseg = 0;     // z-planes per CTA of the ring-pipelined half-sweeps (0: chosen per launch)
    unsigned wait_limit = 1u << 26;   // polls of a ring-pipelined half-sweep's waits before it gives up
    uint32_t pipe_attr = 0;    // pipelined kernel variants whose shared-memory limit is set

    // timing
    std::vector<TimedCall> pending, ev_pool;
    cudaEvent_t marks[8] = {};
    double t_ms = 0;
    long long t_launches = 0, t_updates = 0;

    ResidentTables res;
    std::vector<uint8_t> list_seen;   // scratch of the chain-list checks
};

// ---- error reporting ----
int set_error(int code, const char* fmt, ...);
int cuda_check(cudaError_t e, const char* what);

// Device allocations of one call, freed when the scope ends (error returns included).
struct DeviceScratch {
    std::vector<void*> ptrs;
    template <typename T>
    cudaError_t alloc(T** out, size_t bytes) {
        void* q = nullptr;
        const cudaError_t e = cudaMalloc(&q, bytes);
        if (e == cudaSuccess) {
            ptrs.push_back(q);
            *out = static_cast<T*>(q);
        }
        return e;
    }
    DeviceScratch() = default;
    DeviceScratch(const DeviceScratch&) = delete;
    DeviceScratch& operator=(const DeviceScratch&) = delete;
    ~DeviceScratch() {
        for (void* q : ptrs) cudaFree(q);
    }
};
#define NMMC_CUDA(call)                                         \
    do {                                                        \
        cudaError_t _e = (call);                                \
        if (_e != cudaSuccess) return cuda_check(_e, #call);    \
    } while (0)

// ---- general interaction tables (nmmc_general.cu) ----
int launch_colour_sweeps(Ctx& c, const int* d_chains, int n, int nsweeps);
int launch_energy_general(Ctx& c, const int* d_chains, int n, int rows, int nblk_slice, int nblk_total,
                          double* partial);
int launch_delta_e_general(Ctx& c, int chain, const int32_t* d_sites, const float* d_trial, int n, double* d_out);
int upload_general(Ctx& c);   // (re)writes the device records from h_gje and the DMI sign

// ---- kernels (nmmc_kernels.cu) ----
// fused: the last sweep's half-sweeps also sum E, M, subM and sub4M (hbm_fused_measure_ok);
// launch_measure_fused_tail then finishes the observables.
int launch_global_sweeps(Ctx& c, const int* d_chains, int n, int nsweeps, bool fused = false);
bool hbm_fused_measure_ok(const Ctx& c);
int launch_measure_fused_tail(Ctx& c, const int* d_chains, int n, int accumulate);
int launch_measure(Ctx& c, const int* d_chains, int n, int accumulate);
// nsweeps HBM-path sweeps of every chain and, with `measure`, the observables as
// nmmc_sweep_measure takes them on that path (the autotuner's HBM candidate)
int hbm_tuning_step(Ctx& c, int nsweeps, bool measure);
int measure_prepare(Ctx& c, int n);
size_t measure_partials_per_chain(const Ctx& c);   // partial-sum doubles one chain's measurement uses
int launch_measure_into(Ctx& c, const int* d_chains, int n, double* scratch, size_t scratch_doubles,
                        double* obs, double* q);
int launch_init_spins(Ctx& c);
int launch_add_av(Ctx& c);   // adds the av chains' spins to their sums (no-op without a list)
int launch_delta_e(Ctx& c, int chain, const int32_t* d_sites, const float* d_trial, int n, double* d_out);
int launch_replay(Ctx& c, int chain, const nmmc_event* d_ev, size_t n, uint8_t* d_acc, long long* d_first);
int launch_advance(Ctx& c, const int* d_chains, int n, int nsweeps);

// ---- wavefront sweeps (nmmc_wave.cu) ----
// Tile rows of the wavefront sweep on this lattice (0: the lattice is not covered).
int wave_rows(const Ctx& c);
// One full sweep of the listed chains from src to dst (Philox sweep offset `off`).
int launch_wave_sweep(Ctx& c, const float* src, float* dst, const int* d_chains, int n, unsigned off);
bool wave_ready(Ctx& c);   // nmmc_kernels.cu
// ---- prefetching four-site half-sweep (nmmc_pf.cu) ----
int launch_pf_half(Ctx& c, const int* d_chains, int n, int colour, unsigned off);
long long global_sweep_launches(Ctx& c, int nsweeps, bool fused);

// ---- stencil resident kernel (nmmc_stencil.cu) ----
size_t stencil_chain_bytes(const Ctx& c);   // 0: the lattice is not covered
int stencil_slots(const Ctx& c, int n);     // chains per CTA for a call on n chains (0: none fits)
int launch_stencil_sweeps(Ctx& c, const int* d_chains, int n, int nsweeps, bool measure, int accumulate);

// ---- resident kernel (nmmc_resident.cu) ----
int resident_prepare(Ctx& c);
// all: the list is every chain in order. measure: after the sweeps, compute the listed
// chains' observables in the same launch (2-D lattices; see resident_can_measure).
int launch_resident_sweeps(Ctx& c, const int* d_chains, int n, int nsweeps, bool all, bool measure,
                           int accumulate);
bool resident_can_measure(const Ctx& c);
// The sweeps of this context run on the resident path (after resident_prepare): the option,
// eligibility, and on the automatic path the autotuner's choice between the two paths.
bool resident_chosen(const Ctx& c);
void resident_free(Ctx& c);
// Compact form of masked Heisenberg lattices on the HBM path: allocates and builds the tables
// of every chain when the sweeps will use it (a no-op otherwise or when built); and rebuilds
// one chain's table after its mask changed.
int compact_prepare(Ctx& c);
// compact_table_chain's result when the packed table is in use and one of the chain's
// neighbour differences does not fit in 16 bits (nothing uploaded); otherwise a status code.
constexpr int kTableDoesNotFit = 1;
int compact_table_chain(Ctx& c, int chain);
// Kernel launches of one resident call of nsweeps sweeps.
int resident_launches(const Ctx& c, int nsweeps);

int upload_params(Ctx& c);
void classify_dmi(DevModel& m);
int sweep_impl(Ctx& c, const int* d_chains, const int* h_chains, int n, int nsweeps, bool allow_timing);
int sweep_measure_impl(Ctx& c, const int* d_chains, const int* h_chains, int n, int nsweeps, int accumulate,
                       bool allow_timing);
int resolve_timing(Ctx& c);

}  // namespace nmmc
