/*
 * nmmc.h — C ABI of the GB300 Metropolis spin-lattice sampler.
 *
 * This is the drop-in boundary for NanoMagMC's hot path (waterswims/NanoMagMC, directory
 * Old/). The reference has no plugin or FFI layer: its hot path sits behind the C++ class
 * `state` (Old/includes/state.hpp:12-52) over `particle::td::functionObject`
 * (Old/includes/thermodynamics.hpp:10-85), configured by `stateOptions`/`simOptions`
 * (Old/includes/param_read.hpp:6-37) and driven by Old/lib/main.cpp:104-275. Each entry
 * point below names the reference interface it replaces.
 *
 * Conventions
 *   - Every function returns a status: 0 on success. 103, 104, 105 and 207 keep the
 *     reference's exit-code meanings (bad shape, T <= 0, input file/key missing, bad
 *     protocol); the other codes are listed below. nmmc_last_error() gives a message.
 *   - A context owns all device memory it uses; host buffers belong to the caller.
 *   - One context per host thread; calls are ordered on the context's CUDA stream and the
 *     calls that return host data synchronise that stream.
 *   - Spin arrays exchanged with the host are FP64, three components per site, in box
 *     order (x fastest: index x + E*(y + E*z), E = lattice edge); Ising spins use
 *     component 0 (Old/lib/field_type.cpp:84-93), sites outside the particle hold 0.
 */
#ifndef NMMC_H
#define NMMC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------------- */
#define NMMC_OK 0
#define NMMC_ERR_SHAPE 103       /* Old/lib/state.cpp:76-78            */
#define NMMC_ERR_TEMP 104        /* Old/lib/state.cpp:263-268          */
#define NMMC_ERR_INPUT 105       /* Old/lib/param_read.cpp:12-16,31-32 */
#define NMMC_ERR_PROTOCOL 207    /* Old/lib/protocol.cpp:55-57         */
#define NMMC_ERR_ARG 300         /* bad argument (null pointer, index out of range, size) */
#define NMMC_ERR_UNSUPPORTED 301 /* interaction set or lattice the kernels do not cover   */
#define NMMC_ERR_CUDA 302        /* a CUDA runtime call failed                            */
#define NMMC_ERR_TIMEOUT 303     /* a bounded device-side wait gave up                    */
#define NMMC_ERR_NOMEM 304       /* device or host allocation failed                      */
#define NMMC_ERR_IO 305          /* output file could not be written                      */

#define NMMC_MAX_PATH 256
#define NMMC_MAX_OFFSETS 2048   /* interaction records per table (the FePt tables hold up to 1358) */

/* ---- options: stateOptions + simOptions (Old/includes/param_read.hpp:6-37) ----------- */
typedef struct {
    /* stateOptions */
    double size;         /* SIZE / per-lattice draw (Weibull scale radius)            */
    double edge_size;    /* derived as in Old/lib/param_read.cpp:55-70 (a double)    */
    int is_perio;        /* ISPERIO   */
    int is_ising;        /* ISISING   */
    char shape_code;     /* LATTSHAPE: s/S square, c/C cube, w/W 2-D Weibull, x/X 3-D Weibull */
    double J;            /* EXCHANGE  */
    double K;            /* DMISTREN  */
    double H;            /* initial field (the reference leaves it unset; 0 here)    */
    double k_b;          /* BOLTZMANN */
    double T;            /* initial temperature                                      */
    double beta_w;       /* WEIBULLFACT */
    char int_file[NMMC_MAX_PATH];   /* INTERACTIONS (file name under Js/) */
    /* simOptions */
    char temp_file[NMMC_MAX_PATH];  /* TEMPNAME  (under Temps/)  */
    char field_file[NMMC_MAX_PATH]; /* FIELDNAME (under Fields/) */
    char out_file[NMMC_MAX_PATH];
    int samp_sweeps;     /* SAMPSWEEPS */
    int n_samp;          /* NSAMPS     */
    int eq_sweeps;       /* EQSWEEPS   */
    int n_latts;         /* NLATTS     */
    int protocol;        /* PROTOCOL   */
    int distrib;         /* ISDISTRIB  */
    double amean, asd;   /* MEANSIZE/SIZEDEV, or SIZE and 0 */
    double lmean, lsd;   /* log-normal parameters (AtoLn, Old/lib/functions.cpp:56-62) */
} nmmc_options;

/* Interaction table: one record per line of a Js/ file (Old/lib/field_type.cpp:39-73),
 * already scaled by EXCHANGE (J) and DMISTREN (D). Any offsets: tables of the 2*dim axis
 * neighbours run on the two-colour checkerboard kernels; any other coupling (next-nearest,
 * longer range) runs on the multi-colour gather sweep (see nmmc_colouring). */
typedef struct {
    int dim;
    int n;
    int offset[NMMC_MAX_OFFSETS][3];
    double J[NMMC_MAX_OFFSETS];
    double D[NMMC_MAX_OFFSETS][3];
} nmmc_interactions;

/* One chain = one `state`: its particle realisation, size, temperature and field.
 * Chains with the same `lattice` index and size get the same shape draw, so a chain and
 * its forks (curr_state = base_state) share one particle. */
typedef struct {
    int lattice;
    double size;
    double T;
    double H;
} nmmc_chain_desc;

/* Per-chain observables written by nmmc_measure, NMMC_OBS_N doubles per chain, in this
 * order (Old/lib/main.cpp:185-224): */
enum {
    NMMC_OBS_E = 0,           /* energy()                                   */
    NMMC_OBS_M = 1,           /* magnetisation() components 0..2 (1,2,3)    */
    NMMC_OBS_ABSM = 4,        /* norm(M)                                    */
    NMMC_OBS_SUBM = 5,        /* submag(0) components (5,6,7)               */
    NMMC_OBS_ABSSUBM = 8,
    NMMC_OBS_SUB4M = 9,       /* sub4mag() components (9,10,11)             */
    NMMC_OBS_ABSSUB4M = 12,
    NMMC_OBS_QTOT = 13,       /* sum over slices of tcharge()               */
    NMMC_OBS_N = 14
};

/* Running FP64 accumulators per chain (for specific heat and susceptibility):
 * count, sum E, sum E^2, sum |M|, sum |M|^2, sum |M|^4, sum Q, sum Q^2. */
#define NMMC_ACC_N 8

/* Lattice facts of a context. */
typedef struct {
    int dim, edge, is_ising, is_perio;
    int nchains;
    int nslices;          /* tcharge() length: edge in 3-D, 1 in 2-D */
    long long box_sites;  /* edge^dim */
    char shape_code;
} nmmc_info;

/* One attempt of a sequential random-site chain (the oracle writes these). */
typedef struct {
    int32_t site_box;     /* box index of the chosen site      */
    int32_t accepted;     /* the producer's accept decision    */
    double trial[3];      /* proposed spin                     */
    double u;             /* acceptance uniform (unused if dE <= 0) */
    double dE;            /* the producer's dE                 */
} nmmc_event;

/* Options for nmmc_set_option. */
enum {
    NMMC_OPT_SWEEP_PATH = 1,   /* 0 auto, 1 HBM-streaming half-sweeps, 2 shared-memory resident */
    NMMC_OPT_DMI_SIGN = 2,     /* 0 as the reference's dE (s_j x D), 1 consistent with E (D x s_j) */
    NMMC_OPT_MEASURE_FP64 = 3, /* 1: per-site terms of nmmc_measure in FP64 (default 0: FP32 terms, FP64 sums) */
    NMMC_OPT_PERIODIC_Q = 4,   /* 1: topological-charge triangles wrap on periodic lattices (default 0, as the reference) */
    NMMC_OPT_TIMING = 5,       /* 1: time sweep kernels with CUDA events (see nmmc_get_timing) */
    NMMC_OPT_RESIDENT_THREADS = 6, /* threads per CTA of the resident kernel (0: autotuned) */
    NMMC_OPT_RESIDENT_BINS = 7,    /* number of CTAs (bins) of the resident kernel (0: autotuned) */
    NMMC_OPT_HALF_KERNEL = 8,      /* HBM path: 0 four sites per thread where the lattice allows (3 CTAs/SM),
                                      1 one site per thread, 2 four sites per thread at 2 CTAs/SM;
                                      3-7 the ring-pipelined kernels (3-D periodic lattices of edge 128: the
                                      other colour's planes staged in shared memory by bulk copies issued a
                                      step ahead): 3 tiles of 8 rows and a ring of 4 planes, 4 16 rows and 4
                                      planes, 5 8 rows and 5 planes, 6 and 7 a producer warp and consumer
                                      warps (8 rows, rings of 4 and 5); 8 four sites per thread with the
                                      next quad's spins prefetched into shared memory by cp.async while
                                      the current quad is computed (2 CTAs/SM). All give the same chain */
    NMMC_OPT_COLOURS = 9,          /* read only: colour classes (launches) per sweep; 2 = checkerboard */
    NMMC_OPT_MEASURE_SITES = 10,   /* HBM-path measurement: same-colour sites per thread item, 2 (default) or 4;
                                      the same terms summed in another FP32 order */
    NMMC_OPT_RESIDENT_PREDRAW = 11, /* 2-D resident path: 0 autotuned, 1 off, 2 on where it fits: a separate
                                      kernel computes the Philox words of the coming sweeps on every SM, the
                                      resident kernel reads them (same chain bit for bit); pays when the
                                      chains occupy few SMs. Reads back 1 or 2 once the shape is chosen */
    NMMC_OPT_WAIT_LIMIT = 13,      /* polls of each bounded wait of the ring-pipelined half-sweeps before they
                                      give up (default 2^26; a give-up is reported by nmmc_synchronize as
                                      NMMC_ERR_TIMEOUT, after the kernel has let its copies in flight land) */
    NMMC_OPT_RING_ZSEG = 14,       /* z-planes per CTA of the ring-pipelined half-sweeps (0: chosen per launch) */
    NMMC_OPT_L2_PREFETCH = 15,     /* four-site half-sweeps: each block asks L2 for the spins of the block this
                                      many quarter waves of resident blocks later (default 2; 0: off); the same
                                      chain */
    NMMC_OPT_RESIDENT_STENCIL = 17, /* resident path, unmasked 2-D Heisenberg lattices: 0 autotuned, 1 off, 2 on:
                                      whole chains in shared memory in their split-colour layout, four sites
                                      per thread item with 16-byte loads of the neighbour rows (instead of
                                      per-site neighbour records); the same chain */
    NMMC_OPT_WAVE = 16,            /* HBM path, 3-D unmasked Heisenberg lattices with the checkerboard's axis
                                      tables: 1 runs pairs of sweeps as wavefront launches (both colours of a
                                      sweep in one pass, out of place between the spin array and a second one
                                      allocated at the first such call: every spin read and written once per
                                      sweep), 0 (default) half-sweeps only; the same chain. On the 128^3
                                      benchmark lattices the wavefront sweep moves a third of the bytes but
                                      runs slower (1.26e11 against 1.53e11 updates/s) */
    NMMC_OPT_CHARGE_PASS = 18,     /* nmmc_sweep_measure on the HBM four-site path, the topological-charge pass
                                      after the fused half-sweep: 0 (default) threads walk strips of four
                                      sites along y with three rows in registers (every spin loaded about
                                      once), 1 the measurement kernel's charge-only items; the same
                                      triangles and angles, summed in another FP32 order */
    NMMC_OPT_MASKED_COMPACT = 12   /* masked Heisenberg lattices on the HBM path: 0 (default) sweep the filled
                                      sites in compact planes with neighbour tables (gathered from and written
                                      back to the box layout by each call), 1 sweep them in the box layout over
                                      the filled-site lists; the same chains */
};

typedef struct nmmc_ctx nmmc_ctx;

/* ---- host-side configuration (no GPU) ------------------------------------------------ */

/* read_all_vars (Old/lib/param_read.cpp:35-82): same keys; returns 105 on a missing file
 * or key instead of exiting. Also fills lmean/lsd when ISDISTRIB is set. */
int nmmc_read_input(const char* path, nmmc_options* out);

/* load_Hs_Ts (Old/lib/param_read.cpp:84-151): reads <dir>/Temps/<TEMPNAME> and
 * <dir>/Fields/<FIELDNAME> as whitespace-separated numbers (stored as float, as the
 * reference does). n_T/n_H receive the counts; at most cap values are written. */
int nmmc_load_lists(const nmmc_options* opt, const char* dir, double* Ts, int cap_T, int* n_T,
                    double* Hs, int cap_H, int* n_H);

/* field_type constructor's Js/ reader (Old/lib/field_type.cpp:39-73). */
int nmmc_read_interactions(const char* path, int dim, double J_mod, double D_mod,
                           nmmc_interactions* out);

/* The parallel update order a context with this table uses (no counterpart in the reference,
 * whose sweep is sequential, Old/lib/state.cpp:171-203). out[0] = kind: 0 the two-colour
 * checkerboard (axis nearest-neighbour tables), 1 colour = (x + b*y + c*z) mod q, 2 colour =
 * (x mod p) + p*(y mod p) [+ p*p*(z mod p)]; out[1] = colour classes; out[2] = q or p;
 * out[3] = b; out[4] = c. No two sites of one class interact through any coupling record, and
 * on periodic lattices the period divides the edge. 301 when no colouring of at most 4096
 * classes exists. */
int nmmc_colouring(int dim, int edge, int is_perio, int is_ising, const nmmc_interactions* inter, int out[5]);

/* set_protocol (Old/lib/protocol.cpp:6-59): which list is v1/v2 and the loop bounds.
 * v1_is_T = 1 when v1 runs over temperatures. Returns 207 for an unknown protocol. */
int nmmc_protocol_plan(int protocol, int n_H, int n_T, int* v1_is_T, int* v1_begin,
                       int* v1_end, int* v1_step, int* v2_begin, int* v2_end, int* v2_step);

/* Log-normal particle size for lattice k (std_lognormrand, Old/includes/stdrand.hpp:122-144;
 * main.cpp:116), drawn from Philox keyed by seed. */
double nmmc_lognormal_size(uint64_t seed, int k, double lmean, double lsd);

/* Shape of lattice realisation `lattice` (shape::check, Old/lib/shape.cpp:40-58, applied at
 * every box site as in state::init_lattice, Old/lib/state.cpp:132-153): 1 = filled. For
 * square/cube shapes every site is filled. mask: edge^dim bytes in box order. Writes the
 * site counts num/snum/s4num (Old/lib/state.cpp:136-151) when the pointers are not NULL. */
int nmmc_shape_mask(char shape_code, int edge, double size, double weibull_beta, uint64_t seed,
                    int lattice, uint8_t* mask, int* num, int* snum, int* s4num);

/* Binning analysis of a sample series: mean, its standard error from the plateau of the
 * binned error, and the integrated autocorrelation time estimate. */
int nmmc_binning(const double* x, int n, double* mean, double* err, double* tau);

/* ---- context (replaces `state`) ----------------------------------------------------- */

/* state(stateOptions) x nchains (Old/lib/state.cpp:15-35,48-82,124-169): builds the
 * lattices (shape masks from seed), draws random starting spins, sets T and H per chain.
 * Returns 103 for an unknown shape code, 104 for T <= 0, 301 for interactions the
 * checkerboard kernels do not cover, 300 for more than NMMC_MAX_CHAINS chains. */
#define NMMC_MAX_CHAINS 65535   /* chains per context (the launches put the chain list on grid.y) */
int nmmc_create(const nmmc_options* opt, const nmmc_interactions* inter,
                const nmmc_chain_desc* chains, int nchains, uint64_t seed, nmmc_ctx** out);

/* Destructor (state::~state, Old/lib/state.cpp:119-122). */
void nmmc_destroy(nmmc_ctx* ctx);

int nmmc_get_info(const nmmc_ctx* ctx, nmmc_info* info);

/* num_spins / sub_num / sub4_num (Old/lib/state.cpp:248-261): filled-site counts. */
int nmmc_site_counts(const nmmc_ctx* ctx, int chain, int* num, int* snum, int* s4num);

/* change_temp + change_field (Old/lib/state.cpp:263-276). 104 if T <= 0; the field goes to
 * component 0 for Ising and 2 for Heisenberg spins. */
int nmmc_set_point(nmmc_ctx* ctx, int chain, double T, double H);
int nmmc_set_points(nmmc_ctx* ctx, const int* chains, const double* T, const double* H, int n);
/* The chain's current temperature and field (the scalars `state` keeps, state.hpp:15-18). */
int nmmc_get_point(const nmmc_ctx* ctx, int chain, double* T, double* H);

/* change_v1 / change_v2 (Old/lib/state.cpp:298-326). */
int nmmc_change_v1(nmmc_ctx* ctx, int chain, int protocol, double v1);
int nmmc_change_v2(nmmc_ctx* ctx, int chain, int protocol, double v2);

/* curr_state = base_state (Old/lib/main.cpp:164; Old/lib/state.cpp:84-117): copies spins,
 * T and H of src into dst. dst keeps its own random stream. */
int nmmc_fork(nmmc_ctx* ctx, int src_chain, int dst_chain);

/* equil(nsweeps * N) (Old/lib/state.cpp:171-203) for the listed chains (NULL: all), as
 * nsweeps two-colour checkerboard sweeps. The first sweep call of a context (and the first
 * after an option that changes the resident shape) builds the path's tables on the device
 * (the resident kernel's site tables and autotuning, the compact form of masked lattices):
 * make it outside any stream capture (nmmc_sample prepares them before it captures). */
int nmmc_sweep(nmmc_ctx* ctx, const int* chains, int n, int nsweeps);

/* magnetisation / energy / submag(0) / sub4mag / tcharge (Old/lib/state.cpp:205-246,
 * Old/lib/thermodynamics.cpp:71-221) for the listed chains (NULL: all). obs receives
 * NMMC_OBS_N doubles per chain; q (may be NULL) receives nslices doubles per chain.
 * accumulate != 0 also adds the sample to the chain's FP64 accumulators. With obs == NULL
 * (and q == NULL) the call only enqueues the measurement: results stay on the device and
 * reach the host through nmmc_get_accumulators. */
int nmmc_measure(nmmc_ctx* ctx, const int* chains, int n, double* obs, double* q, int accumulate);

/* Allocation-free measurement, for callers that cannot call cudaMalloc: code running while
 * a CUDA stream is being captured (allocation is refused during capture), frameworks that
 * give out device memory only from their own pool, and latency-critical loops that cannot
 * afford cudaMalloc's implicit device synchronisation. No counterpart in the reference.
 *
 * Same observables as nmmc_measure (no accumulation), from the same kernels with the same
 * block split, written to caller-owned DEVICE memory: d_obs receives NMMC_OBS_N doubles per
 * chain, d_q (may be NULL) nslices doubles per chain. d_chains is a device array of n chain
 * indices, or NULL for all chains; an entry outside [0, nchains) is not read and its rows of
 * d_obs and d_q are NaN; entries may repeat; n = 0 does nothing. The call only enqueues work
 * on the context's stream (nmmc_stream), after one copy of changed (T, H) values from the
 * context's page-locked staging block; synchronise before reading.
 *
 * The kernels' partial sums live in one fixed device array of NMMC_STATIC_SCRATCH_DOUBLES
 * doubles (2 MiB) that every GPU loading the library holds until exit. One chain needs 11
 * doubles per measurement block: blocks = slices x ceil(edge / max(1, 4096 / edge)) on
 * unmasked lattices (a 128^3 lattice: 512 blocks, 5632 doubles, so 46 chains per call),
 * slices x ceil(filled sites of the fullest slice / 4096) on masked ones; a device list
 * adds n / 2 doubles (rounded up to a multiple of 32). Larger requests are rejected with
 * NMMC_ERR_ARG, whose message gives the lattice's limit. The array is shared by every call in
 * the process and keeps the last call's contents; each call writes every slot it reads, so
 * nothing needs clearing, but calls that overlap on the GPU (other streams or contexts) race
 * on it. The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) with that device current; make that first call before any stream
 * capture. */
#define NMMC_STATIC_SCRATCH_DOUBLES 262144
int nmmc_measure_static(nmmc_ctx* ctx, const int* d_chains, int n, double* d_obs, double* d_q);

/* One sample step of Old/lib/main.cpp:207-231: equil(nsweeps * N) then energy(),
 * magnetisation(), submag(0), sub4mag(), tcharge() of the listed chains (NULL: all); outputs
 * and accumulation as nmmc_measure. Chains are identical to nmmc_sweep followed by
 * nmmc_measure. On the shared-memory resident path of a 2-D lattice the observables are
 * computed by the sweep launch itself from the spins it holds on chip. On the HBM path's
 * four-site kernel (unmasked Heisenberg lattices whose +-axis records are pairs, FP32
 * observables) the last sweep's colour-1 half-sweep sums E, M, submag and sub4mag on the way
 * (every bond joins the two colours, and colour 0 is final by then) and one pass over the
 * lattice adds the charge (NMMC_OPT_CHARGE_PASS). In both cases the FP32 per-site terms are
 * summed in another order than nmmc_measure's, so values agree to FP32 rounding rather than
 * bit for bit (every solid angle is the same FP32 value, summed in another order).
 * Elsewhere the call is nmmc_sweep + nmmc_measure. */
int nmmc_sweep_measure(nmmc_ctx* ctx, const int* chains, int n, int nsweeps, double* obs, double* q,
                       int accumulate);

/* nsamples x nmmc_sweep_measure(nsweeps, accumulate = 1), replayed as one CUDA graph per
 * sample, for the inner sampling loop of Old/lib/main.cpp:182-240.
 * obs: nsamples x n x NMMC_OBS_N, q: nsamples x n x nslices (may be NULL). */
int nmmc_sample(nmmc_ctx* ctx, const int* chains, int n, int nsweeps, int nsamples,
                double* obs, double* q);

/* FP64 accumulators: NMMC_ACC_N doubles per listed chain. */
int nmmc_get_accumulators(nmmc_ctx* ctx, const int* chains, int n, double* out);
int nmmc_reset_accumulators(nmmc_ctx* ctx);

/* Spins in and out (field_type::print / set_spin). n_sites = box sites; xyz holds 3 doubles
 * per box site, x fastest (Ising: component 0). */
int nmmc_get_spins(nmmc_ctx* ctx, int chain, double* xyz, size_t n_sites);
int nmmc_set_spins(nmmc_ctx* ctx, int chain, const double* xyz, size_t n_sites);

/* Summed lattices (state::add_to_av, Old/lib/state.cpp:288-296, called after every sample at
 * Old/lib/main.cpp:236-239): the listed chains' spins are added, in FP64 on the device, to a
 * per-chain sum at every accumulating measurement (nmmc_measure or nmmc_sweep_measure with
 * accumulate != 0, and every sample of nmmc_sample). Setting the list zeroes the sums
 * (summed_field.all_zero(), main.cpp:177); n = 0 stops summing. */
int nmmc_set_av_chains(nmmc_ctx* ctx, const int* chains, int n);
/* The sum of one listed chain, in nmmc_get_spins's layout. */
int nmmc_get_av(nmmc_ctx* ctx, int chain, double* xyz, size_t n_sites);
/* 1 where the box site belongs to the particle (shape::check), 0 elsewhere. */
int nmmc_get_mask(nmmc_ctx* ctx, int chain, uint8_t* mask, size_t n_sites);

/* calc_dE (Old/lib/thermodynamics.cpp:51-69) on the device for n proposals at box sites,
 * with the FP32 arithmetic of the sweep kernels; dE written as double. */
int nmmc_delta_e(nmmc_ctx* ctx, int chain, const int32_t* sites, const double* trial, int n,
                 double* dE);

/* Sequential replay: applies n logged attempts to one chain in order, in FP64, with the
 * reference's dE and acceptance rule (Old/lib/state.cpp:180-202). accepted[i] receives
 * this replay's decision; *first_mismatch the first index whose decision differs from
 * the log (-1 if none); final_xyz (may be NULL) the FP64 spins after the replay. The
 * chain's FP32 spins are overwritten with the result. No reference counterpart. */
int nmmc_debug_replay(nmmc_ctx* ctx, int chain, const nmmc_event* events, size_t n,
                      uint8_t* accepted, int64_t* first_mismatch, double* final_xyz);

int nmmc_set_option(nmmc_ctx* ctx, int key, int64_t value);
int nmmc_get_option(const nmmc_ctx* ctx, int key, int64_t* value);

/* Sweep-kernel time recorded with CUDA events while NMMC_OPT_TIMING is 1: total ms,
 * number of kernel launches and of site updates attempted. Reading resets the totals. */
int nmmc_get_timing(nmmc_ctx* ctx, double* ms, long long* launches, long long* updates);

/* CUDA-event markers on the context's stream: nmmc_timer_mark records event `slot`
 * (0..7); nmmc_timer_elapsed waits for slot b and returns the device time from a to b. */
int nmmc_timer_mark(nmmc_ctx* ctx, int slot);
int nmmc_timer_elapsed(nmmc_ctx* ctx, int slot_a, int slot_b, double* ms);

/* The context's CUDA stream (a cudaStream_t), for callers that order their own work. */
/* Page-locked host memory (cudaHostAlloc) for callers' per-step inputs and outputs, so that
 * the library's copies to and from them run asynchronously at full bus speed. No counterpart
 * in the reference. */
int nmmc_host_alloc(size_t bytes, void** out);
int nmmc_host_free(void* p);

void* nmmc_stream(nmmc_ctx* ctx);
/* Waits for the context's stream; NMMC_ERR_TIMEOUT if a pipelined kernel's bounded wait gave up. */
int nmmc_synchronize(nmmc_ctx* ctx);

/* Message of the last failed call on this thread. */
const char* nmmc_last_error(void);

/* ---- learned warm start (no reference counterpart) ------------------------------------ *
 * A conditional convolutional generator for unmasked 2-D Heisenberg lattices of edge L
 * (a multiple of 16): 8 periodic 3x3 convolutions of 48 channels, BF16 weights and
 * activations, FP32 accumulation. It is trained on equilibrium snapshots that the sampler
 * itself produced, to denoise y = normalise(sqrt(1-s^2) x + s g) back to the snapshot x;
 * at s = 1, y is a uniform random start. Conditions are (T, B, D) per snapshot. */
typedef struct nmmc_gen nmmc_gen;

/* capacity: number of snapshots the dataset can hold. Weights from Philox(seed). */
int nmmc_gen_create(int L, int capacity, uint64_t seed, nmmc_gen** out);
void nmmc_gen_destroy(nmmc_gen* gen);
int nmmc_gen_param_count(const nmmc_gen* gen);
/* FP32 master parameters in layer order: W[9][cin][cout] (tap = 3*(dy+1)+(dx+1)), then b[cout];
 * the first layer has cin = 8 (y, T/1.5, B, D/0.8, s, 0), the last cout = 4 (3 + 1 zero). */
int nmmc_gen_get_params(nmmc_gen* gen, float* out, int n);
int nmmc_gen_set_params(nmmc_gen* gen, const float* in, int n);
/* Copies the current spins of the listed chains (with their (T, B, D) in cond[3n]) into the
 * dataset, on the device. */
int nmmc_gen_add_snapshots(nmmc_gen* gen, nmmc_ctx* ctx, const int* chains, int n, const double* cond);
int nmmc_gen_dataset_size(const nmmc_gen* gen);
/* One Adam step on a batch (snapshot indices idx[nb], noise levels sig[nb]); *loss = mean
 * |v/|v| - x|^2 per site. lr <= 0 computes loss and gradients only. */
int nmmc_gen_train_step(nmmc_gen* gen, const int* idx, const float* sig, int nb, float lr, double* loss);
/* Gradients of the last step and its network input ([nb][L][L][8]), for checks. */
int nmmc_gen_get_grads(nmmc_gen* gen, float* out, int n);
int nmmc_gen_get_input(nmmc_gen* gen, int nb, float* out);
/* Warm start: `steps` denoising passes from a uniform random start at s = 1 - k/steps,
 * written into the listed chains' spins; cond[3n] = (T, B, D) per chain. Between passes
 * the estimate is re-noised to the next level with fresh noise (reuse_noise = 0), with
 * the noise the network's estimate implies (reuse_noise = 1, a DDIM-style update), or by the
 * variance-preserving posterior step from the previous noisy state (reuse_noise = 2, a
 * DDPM-style update). */
int nmmc_gen_warm_start(nmmc_gen* gen, nmmc_ctx* ctx, const int* chains, int n, const double* cond, int steps,
                        int reuse_noise);
/* Statistics of long plain chains, the reference a warm start is judged against: eq_sweeps
 * sweeps of the listed chains, then nsamp samples gap sweeps apart (nmmc_sample, so they are
 * added to the chains' accumulators). out[3k .. 3k+2] for k = E/N, |M|/N, Q: the mean, one
 * chain's spread and the standard error of the mean from the per-chain averages. */
int nmmc_reference_stats(nmmc_ctx* ctx, const int* chains, int n, int eq_sweeps, int nsamp, int gap,
                         double out[9]);
/* The warm start with its gate and fallback: `steps` denoising passes into the listed chains
 * (nmmc_gen_warm_start, DDPM-style), check_sweeps plain sweeps, then nsamp samples gap sweeps
 * apart. The learned start is kept (*kept = 1) when E/N, |M|/N and Q agree within 3 standard
 * errors of the difference with ref (nmmc_reference_stats of long plain chains) or, with ref
 * NULL, with the same chains' next nsamp samples (a drift test). Otherwise the chains are
 * restarted from uniform random spins drawn from `seed` (the reference's start,
 * Old/lib/field_type.cpp:197-204) and *kept = 0. The samples are added to the accumulators. */
int nmmc_gen_gated_warm_start(nmmc_gen* gen, nmmc_ctx* ctx, const int* chains, int n, const double* cond, int steps,
                              int check_sweeps, int nsamp, int gap, const double* ref, uint64_t seed, int* kept);
/* Generator options. NMMC_GEN_OPT_TENSOR_CORES: 1 (default) runs the six 48-channel hidden
 * convolutions on the tensor cores (tcgen05.mma, FP32 accumulation in tensor memory; forward
 * in BF16, data gradient in TF32, weight gradient with the FP32 output gradient as BF16 hi + lo
 * operands), with the input windows staged by TMA at L = 128 and by cp.async otherwise. 2: warp-specialised forward with cp.async-staged windows; 3: cp.async
 * staging at every L; 4: at L = 128 a warp-specialised forward (producer, MMA and epilogue
 * warps over a ring of TMA-staged windows); 0: the FP32 FMA pipes. The tensor-core variants
 * give identical results. */
#define NMMC_GEN_OPT_TENSOR_CORES 1
/* NMMC_GEN_OPT_TILE_ROWS: output rows per tile of the TMA-staged forward convolutions at
 * L = 128, 2 (default: one window of four input rows, one commit and one epilogue pass per
 * two rows) or 1; the same results. */
#define NMMC_GEN_OPT_TILE_ROWS 2
/* NMMC_GEN_OPT_WEIGHT_IMAGE: 1 (default) the TMA-staged forward convolutions copy each layer's
 * weights into shared memory as one bulk copy of an image in the tensor-core operand layout
 * (rebuilt whenever the weights change); 0 the threads rearrange the BF16 weights; the same
 * results. */
#define NMMC_GEN_OPT_WEIGHT_IMAGE 3
/* NMMC_GEN_OPT_SCHEDULE: noise levels of the warm start's denoising passes, pass k of K at
 * s = 1 - k/K (0, default), (1 - k/K)^2 (1: more passes at low noise, where the fine
 * structure forms) or cos(pi/2 k/K) (2). */
#define NMMC_GEN_OPT_SCHEDULE 4
int nmmc_gen_set_option(nmmc_gen* gen, int key, int64_t value);
/* Probe: one layer's convolution of caller data — layer 0 (8 -> 48 channels), 1..6 (48 -> 48)
 * or 7 (48 -> 4); in [nimg][L][L][cin] (rounded to BF16), out [nimg][L][L][cout] = conv + bias
 * in FP32, no activation — as the generator runs it on the tensor cores (tensor != 0; the
 * first and last layers only at L = 128) or on the FP32 FMA pipes. */
int nmmc_gen_probe_conv(nmmc_gen* gen, int layer, int nimg, const float* in, float* out, int tensor);
/* Probe: a hidden layer's weight gradient gw[9][48][48] (tap, input channel, output channel) =
 * sum over the images' pixels p of in[p + tap][ci] * dout[p][co], periodic, for caller data
 * in [nimg][L][L][48] (rounded to BF16) and dout [nimg][L][L][48] (FP32): on the tensor cores
 * (tensor != 0, L a multiple of 16 up to 64 or of 64: tcgen05.mma kind::f16 over K-blocks of
 * min(L, 64) pixels of one row, dout as BF16 hi + lo, within about 4e-6 of the FP64 sum
 * relative to the terms' magnitudes) or on the FP32 FMA pipes. */
int nmmc_gen_probe_wgrad(nmmc_gen* gen, int nimg, const float* in, const float* dout, float* gw, int tensor);
int nmmc_gen_save(nmmc_gen* gen, const char* path);
int nmmc_gen_load(nmmc_gen* gen, const char* path);

/* ---- protocol driver (replaces Old/lib/main.cpp) -------------------------------------- */

/* Runs the reference's program for an INPUT file: reads it and the Temps/, Fields/, Js/
 * lists under workdir, builds NLATTS lattices (log-normal sizes if ISDISTRIB), and runs
 * PROTOCOL's v1/v2 loops with the initial 20*EQSWEEPS equilibration, EQSWEEPS per point
 * and NSAMPS samples SAMPSWEEPS apart, on one GPU. Writes the sample arrays of
 * Old/lib/output.cpp:161-249 as .npy files under outdir (shape [nH, nT, NSAMPS*NLATTS],
 * top_chars [nH, nT, nslices, NSAMPS*NLATTS]) and keeps the /Complete resume flags of
 * Old/lib/output.cpp:429-444 in outdir/complete.npy. verbose != 0 prints progress. Two optional
 * keys beyond the reference's: "GENERATOR <file>" (a generator saved by nmmc_gen_save, relative
 * to workdir; 2-D unmasked Heisenberg lattices of the generator's edge) gives the base chains a
 * learned warm start at (Tmax, 0, DMISTREN) behind nmmc_gen_gated_warm_start's drift gate with
 * EQSWEEPS check sweeps; kept, the initial 20*EQSWEEPS are skipped, rejected, the chains are
 * back at random spins and take them. "WSSTEPS <n>" sets the denoising passes (default 32),
 * "WSSCHED <k>" their noise schedule (NMMC_GEN_OPT_SCHEDULE, default 0).
 * outdir/warm_start.npy then holds [kept, passes]. */
int nmmc_run(const char* input_path, const char* workdir, const char* outdir, uint64_t seed,
             int verbose);

#ifdef __cplusplus
}
#endif
#endif /* NMMC_H */
