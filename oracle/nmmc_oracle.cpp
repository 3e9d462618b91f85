// ORACLE — test infrastructure only.
//
// A CPU restatement, in plain C++17 and FP64, of NanoMagMC's Metropolis hot path
// (waterswims/NanoMagMC, directory Old/). Only tests/, the package smoke check and
// bench.py's CPU-baseline leg may load this library; the product never does.
//
// What is restated, with the reference file:line each part follows:
//   * lattice build (raster, shape mask, site counts) ...... Old/lib/state.cpp:124-169
//   * Weibull shape test ................................... Old/lib/shape.cpp:19-26,40-58
//   * interaction-file reader .............................. Old/lib/field_type.cpp:22-74
//   * default spins / all_rand / gen_rand .................. Old/lib/field_type.cpp:76-95,185-204
//   * neighbour lists and the 4 in-plane `adj` entries ..... Old/lib/field_type.cpp:104-183
//   * E, dE, M, subM, sub4M, Q, solid angle ................ Old/lib/thermodynamics.cpp:10-221
//   * random-site Metropolis (state::equil) ................ Old/lib/state.cpp:171-203
//   * cross product ........................................ Old/lib/functions.cpp:70-78
//   * test fixtures gen_fm / gen_afm / gen_skyrm ........... Old/tests/test_functions.hpp:19-128
//
// Deliberate differences (each one is stated where it happens):
//   * neighbour lists are built by direct box lookup (O(N z)) instead of the reference's
//     O(N^2 z) scan; the resulting lists are identical (same offset order, same first match);
//   * the 3-D raster uses the correct odometer, not the one at state.cpp:154-165 (which
//     visits (x, L, 0) and skips (x+1, 0, 0));
//   * random numbers: the reference uses GSL 1.x/2.x MT19937 (gsl_rng_mt19937, version not
//     pinned; libgsl is absent here). The restatement below uses the standard MT19937
//     recurrence with GSL's seeding rule and restates GSL's published algorithms for
//     gsl_rng_uniform, gsl_rng_uniform_int, gsl_ran_dir_3d (Knop's method) and
//     gsl_ran_lognormal (polar Box-Muller). This cannot be checked against GSL here, so the
//     bit-stream is unpinned; only the distributions matter for parity.
//   * the Weibull mask and the checkerboard mode draw from a Philox4x32-10 restatement
//     (Salmon et al., SC'11) keyed exactly like the GPU library, so both sides build the
//     same masks and, for Ising, the same checkerboard chain.
//
// Compiled with -ffp-contract=off so that results do not depend on the host ISA.

#include <array>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <random>
#include <string>
#include <vector>

namespace {

using V4 = std::array<double, 4>;
using I4 = std::array<int, 4>;

// ----------------------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw: "Parallel random numbers: as easy as 1, 2, 3")
// ----------------------------------------------------------------------------------------
void philox10(uint32_t c[4], uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0;
        uint32_t n1 = (uint32_t)p1;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
        uint32_t n3 = (uint32_t)p0;
        c[0] = n0; c[1] = n1; c[2] = n2; c[3] = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

// Stream selectors in counter word 2 (bits 28..31); same layout as the GPU library.
constexpr uint32_t STREAM_SWEEP = 0u, STREAM_MASK = 2u;

// ----------------------------------------------------------------------------------------
// MT19937 streams with GSL's semantics (see header comment).
// ----------------------------------------------------------------------------------------
struct GslLikeMt {
    std::mt19937 mt;
    explicit GslLikeMt(unsigned long seed) { set(seed); }
    void set(unsigned long seed) { mt.seed(seed == 0 ? 4357u : (uint32_t)seed); }  // GSL: 0 -> 4357
    uint32_t raw() { return (uint32_t)mt(); }
    double uniform() { return raw() / 4294967296.0; }                             // [0,1)
    double uniform_pos() { double u; do { u = uniform(); } while (u == 0); return u; }
    // uniform integer in {0,1}: rejection on floor(raw / floor(range / n)), range = 2^32-1
    int uniform_int2() {
        const uint32_t scale = 0xffffffffu / 2u;
        uint32_t k;
        do { k = raw() / scale; } while (k >= 2u);
        return (int)k;
    }
    // uniform direction on S^2 (Knop): (x,y) uniform in the unit disc, s = x^2+y^2,
    // z = 2s - 1, (x,y) scaled by 2 sqrt(1-s).
    void dir3d(double& x, double& y, double& z) {
        double s;
        do {
            x = -1 + 2 * uniform();
            y = -1 + 2 * uniform();
            s = x * x + y * y;
        } while (s > 1.0);
        z = -1 + 2 * s;
        double a = 2 * std::sqrt(1 - s);
        x *= a;
        y *= a;
    }
    // log-normal via the polar method
    double lognormal(double zeta, double sigma) {
        double u, v, r2;
        do {
            u = -1 + 2 * uniform();
            v = -1 + 2 * uniform();
            r2 = u * u + v * v;
        } while (r2 > 1.0 || r2 == 0);
        double normal = u * std::sqrt(-2.0 * std::log(r2) / r2);
        return std::exp(sigma * normal + zeta);
    }
};

struct RngSet {          // the reference's three global generators (main.cpp:15-16, field_type.cpp:20)
    GslLikeMt rint, rdouble, rsphere;
    RngSet(unsigned long si, unsigned long sd, unsigned long ss) : rint(si), rdouble(sd), rsphere(ss) {}
};

// ----------------------------------------------------------------------------------------
// Lattice (field_type + the parts of state that own it)
// ----------------------------------------------------------------------------------------
struct Lattice {
    int d = 2, edge = 0;
    bool ising = false, periodic = false;
    char shape = 's';
    double wsize = 0, wbeta = 0, wr0 = 0;
    std::vector<V4> spins;
    std::vector<I4> locs;
    std::vector<std::vector<int>> neigh, neigh_choice;
    std::vector<I4> adj;
    std::vector<I4> loc_diffs;
    std::vector<double> J_diffs;
    std::vector<V4> D_vecs;
    std::vector<int> box_to_site;   // logical box (x + edge*(y + edge*z)) -> site or -1
    V4 upspin{}, downspin{}, testspin{};
    int snum = 0, s4num = 0;
    bool useJ = true, useD = false;
    int dmi_sign = 0;               // 0: as the reference's dE (s_j x D); 1: consistent (D x s_j)
    V4 H{};
    double beta = 1.0;

    int box_index(const I4& l) const { return l[0] + edge * (l[1] + edge * (d == 3 ? l[2] : 0)); }
};

void set_default_spins(Lattice& L) {       // field_type.cpp:76-95
    L.upspin = {0, 0, 0, 0};
    L.downspin = L.upspin;
    L.testspin = L.upspin;
    int c = L.ising ? 0 : 2;
    L.upspin[c] = 1;
    L.downspin[c] = -1;
}

void add_spin(Lattice& L, const I4& loc) {  // field_type.cpp:97-102
    L.spins.push_back(L.upspin);
    L.locs.push_back(loc);
}

// field_type.cpp:104-183, with a box lookup in place of the O(N^2) scan.
void set_neigh(Lattice& L) {
    const int n = (int)L.spins.size();
    int nbox = L.edge * L.edge * (L.d == 3 ? L.edge : 1);
    L.box_to_site.assign(nbox, -1);
    for (int i = 0; i < n; ++i) {
        const I4& l = L.locs[i];
        bool inside = true;
        for (int k = 0; k < L.d; ++k) inside = inside && l[k] >= 0 && l[k] < L.edge;
        if (inside && L.box_to_site[L.box_index(l)] < 0) L.box_to_site[L.box_index(l)] = i;
    }
    auto find = [&](const I4& t, int self) -> int {
        for (int k = 0; k < L.d; ++k)
            if (t[k] < 0 || t[k] >= L.edge) return -1;
        if (t[3] != 0 || (L.d == 2 && t[2] != 0)) return -1;
        int j = L.box_to_site[L.box_index(t)];
        return (j == self) ? -1 : j;   // the reference skips i == j
    };
    L.neigh.assign(n, {});
    L.neigh_choice.assign(n, {});
    L.adj.assign(n, I4{-1, -1, -1, -1});
    for (int i = 0; i < n; ++i) {
        for (size_t k = 0; k < L.loc_diffs.size(); ++k) {
            I4 t;
            for (int c = 0; c < 4; ++c) t[c] = L.locs[i][c] + L.loc_diffs[k][c];
            if (L.periodic)
                for (int c = 0; c < L.d; ++c) t[c] = (L.edge + (t[c] % L.edge)) % L.edge;
            int j = find(t, i);
            if (j >= 0) {
                L.neigh[i].push_back(j);
                L.neigh_choice[i].push_back((int)k);
            }
        }
        // adj: raw coordinate differences, never wrapped (field_type.cpp:143-181)
        const int dx[4] = {1, -1, 0, 0}, dy[4] = {0, 0, 1, -1};
        for (int a = 0; a < 4; ++a) {
            I4 t = L.locs[i];
            t[0] += dx[a];
            t[1] += dy[a];
            L.adj[i][a] = find(t, i);
        }
    }
}

// Weibull test (shape.cpp:40-58); the uniform comes from Philox keyed by (seed, chain, box).
bool weibull_check(const Lattice& L, const int* pos, double u) {
    double centre = double(L.edge - 1) / 2.;
    double dist2 = 0;
    for (int i = 0; i < L.d; ++i) dist2 += std::pow((pos[i] - centre) / L.wsize, 2);
    double dist = std::pow(dist2, 0.5);
    double test = std::exp(-std::pow((dist / L.wr0), L.wbeta));
    return u < test;
}

double mask_uniform(uint64_t seed, uint32_t chain, uint32_t box) {
    uint32_t c[4] = {box, 0u, STREAM_MASK << 28, chain};
    philox10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    return c[0] * (1.0 / 4294967296.0);
}

// init_lattice (state.cpp:124-169) with the correct odometer; pos[d-1] runs fastest.
void init_lattice(Lattice& L, const uint8_t* mask_in, uint64_t seed, uint32_t chain) {
    L.snum = 0;
    L.s4num = 0;
    const int dim = L.d;
    long total = 1;
    for (int k = 0; k < dim; ++k) total *= L.edge;
    int pos[3] = {0, 0, 0};
    for (long i = 0; i < total; ++i) {
        I4 posva = {pos[0], pos[1], dim == 3 ? pos[2] : 0, 0};
        bool fill = true;
        if (L.shape == 'w' || L.shape == 'W' || L.shape == 'x' || L.shape == 'X') {
            int box = L.box_index(posva);
            if (mask_in) fill = mask_in[box] != 0;
            else fill = weibull_check(L, pos, mask_uniform(seed, chain, (uint32_t)box));
        }
        if (fill) {
            add_spin(L, posva);
            int possum = 0;
            for (int k = 0; k < dim; ++k) possum += pos[k];
            if (possum % 2 == 0) L.snum++;
            int possum2 = posva[0] + posva[1];
            int posdiff = -posva[0] + posva[1] + (L.edge - L.edge % 4);
            if (possum2 % 4 == 0 && posdiff % 4 == 0 && posva[2] % 4 == 0) L.s4num++;
            else if (possum2 % 4 == 2 && posdiff % 4 == 2 && posva[2] % 4 == 2) L.s4num++;
        }
        // correct odometer
        for (int j = dim - 1; j >= 0; --j) {
            if (++pos[j] < L.edge) break;
            pos[j] = 0;
        }
    }
}

void cprod(const V4& a, const V4& b, V4& o) {   // functions.cpp:70-78
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

V4 calc_M(const Lattice& L) {                     // thermodynamics.cpp:99-111
    V4 v{0, 0, 0, 0};
    for (const V4& s : L.spins)
        for (int c = 0; c < 4; ++c) v[c] += s[c];
    return v;
}

double calc_E(const Lattice& L) {                 // thermodynamics.cpp:71-96 (+ :17-40)
    V4 vsum{0, 0, 0, 0};
    const int n = (int)L.spins.size();
    for (int i = 0; i < n; ++i) {
        V4 vt{0, 0, 0, 0};
        for (size_t j = 0; j < L.neigh[i].size(); ++j) {
            const V4& sj = L.spins[L.neigh[i][j]];
            int k = L.neigh_choice[i][j];
            if (L.useJ)
                for (int c = 0; c < 4; ++c) vt[c] += L.J_diffs[k] * sj[c];
            if (L.useD) {
                V4 t2{0, 0, 0, 0};
                cprod(L.D_vecs[k], sj, t2);
                for (int c = 0; c < 4; ++c) vt[c] += t2[c];
            }
        }
        for (int c = 0; c < 4; ++c) vsum[c] += vt[c] * L.spins[i][c];
    }
    V4 m = calc_M(L);
    double res[3];
    for (int c = 0; c < 3; ++c) res[c] = -L.H[c] * m[c] - 0.5 * vsum[c];
    return res[0] + res[1] + res[2];
}

double calc_dE(const Lattice& L, int pos, const V4& trial) {   // thermodynamics.cpp:51-69 (+ :24-28,41-48)
    V4 vdiff, vsum{0, 0, 0, 0};
    for (int c = 0; c < 4; ++c) vdiff[c] = L.spins[pos][c] - trial[c];
    for (size_t j = 0; j < L.neigh[pos].size(); ++j) {
        const V4& sj = L.spins[L.neigh[pos][j]];
        int k = L.neigh_choice[pos][j];
        if (L.useJ)
            for (int c = 0; c < 4; ++c) vsum[c] += L.J_diffs[k] * sj[c];
        if (L.useD) {
            V4 t{0, 0, 0, 0};
            if (L.dmi_sign == 0) cprod(sj, L.D_vecs[k], t);   // as written in the reference
            else cprod(L.D_vecs[k], sj, t);                    // consistent with calc_E
            for (int c = 0; c < 4; ++c) vsum[c] += t[c];
        }
    }
    double res[3];
    for (int c = 0; c < 3; ++c) res[c] = (L.H[c] + vsum[c]) * vdiff[c];
    return res[0] + res[1] + res[2];
}

V4 calc_subM(const Lattice& L, int sub) {         // thermodynamics.cpp:113-136
    V4 v{0, 0, 0, 0};
    for (size_t i = 0; i < L.spins.size(); ++i) {
        int possum = 0;
        for (int j = 0; j < L.d; ++j) possum += L.locs[i][j];
        if (possum % 2 == sub)
            for (int c = 0; c < 4; ++c) v[c] += L.spins[i][c];
    }
    return v;
}

V4 calc_sub4M(const Lattice& L) {                 // thermodynamics.cpp:138-163 (C's truncating %)
    V4 v{0, 0, 0, 0};
    for (size_t i = 0; i < L.spins.size(); ++i) {
        int k = (L.d == 3) ? L.locs[i][2] : 0;
        int possum = L.locs[i][0] + L.locs[i][1];
        int posdiff = -L.locs[i][0] + L.locs[i][1] + (L.edge - L.edge % 4);
        bool in = (possum % 4 == 0 && posdiff % 4 == 0 && k % 4 == 0) ||
                  (possum % 4 == 2 && posdiff % 4 == 2 && k % 4 == 2);
        if (in)
            for (int c = 0; c < 4; ++c) v[c] += L.spins[i][c];
    }
    return v;
}

double solid_angle(const V4& s1, const V4& s2, const V4& s3) {   // thermodynamics.cpp:200-221
    double s1s2 = s1[0] * s2[0] + s1[1] * s2[1] + s1[2] * s2[2];
    double s1s3 = s1[0] * s3[0] + s1[1] * s3[1] + s1[2] * s3[2];
    double s2s3 = s2[0] * s3[0] + s2[1] * s3[1] + s2[2] * s3[2];
    double rho = 2 * (1 + s1s2) * (1 + s1s3) * (1 + s2s3);
    double dotsum = 1 + s1s2 + s1s3 + s2s3;
    V4 t{0, 0, 0, 0};
    cprod(s1, s3, t);
    double crosssum = t[0] * s2[0] + t[1] * s2[1] + t[2] * s2[2];
    return -std::atan2(crosssum / rho, dotsum / rho);
}

std::vector<double> calc_TC(const Lattice& L) {   // thermodynamics.cpp:165-198
    int tcsize = (L.d == 3) ? L.edge : 1;
    std::vector<double> out(tcsize, 0.0);
    for (size_t i = 0; i < L.spins.size(); ++i) {
        const I4& a = L.adj[i];
        int slice = L.locs[i][2];
        if (a[1] >= 0 && a[2] >= 0) out[slice] += solid_angle(L.spins[i], L.spins[a[1]], L.spins[a[2]]);
        if (a[0] >= 0 && a[3] >= 0) out[slice] += solid_angle(L.spins[i], L.spins[a[0]], L.spins[a[3]]);
    }
    for (double& q : out) q /= 2 * M_PI;
    return out;
}

void gen_rand(Lattice& L, RngSet& R) {            // field_type.cpp:185-195
    if (L.ising) L.testspin[0] = R.rint.uniform_int2() * 2 - 1;
    else R.rsphere.dir3d(L.testspin[0], L.testspin[1], L.testspin[2]);
}

struct Event {            // one attempt of the random-site chain
    int32_t site_box;     // logical box index x + edge*(y + edge*z)
    int32_t accepted;
    double trial[3];
    double u;             // acceptance uniform (0 when dE <= 0 and none was drawn)
    double dE;
};
static_assert(sizeof(Event) == 48, "event layout");

// state::equil (state.cpp:171-203)
void equil(Lattice& L, RngSet& R, long iter, Event* log) {
    const int size = (int)L.spins.size();
    for (long i = 0; i < iter; ++i) {
        int choice = int(R.rdouble.uniform() * size);
        gen_rand(L, R);
        double dE = calc_dE(L, choice, L.testspin);
        int acc = 0;
        double u = 0;
        if (dE <= 0) {
            acc = 1;
        } else {
            u = R.rdouble.uniform();
            double log_eta = std::log(u);
            if ((-dE * L.beta) > log_eta) acc = 1;
        }
        if (acc) L.spins[choice] = L.testspin;
        if (log) {
            Event& e = log[i];
            e.site_box = L.box_index(L.locs[choice]);
            e.accepted = acc;
            e.trial[0] = L.testspin[0];
            e.trial[1] = L.testspin[1];
            e.trial[2] = L.testspin[2];
            e.u = u;
            e.dE = dE;
        }
    }
}

// Replay an event log (sites, trial spins, uniforms) through the same dE/acceptance rule.
long replay(Lattice& L, const Event* ev, long n, uint8_t* acc_out) {
    long first_mismatch = -1;
    for (long i = 0; i < n; ++i) {
        int site = L.box_to_site[ev[i].site_box];
        V4 t{ev[i].trial[0], ev[i].trial[1], ev[i].trial[2], 0};
        double dE = calc_dE(L, site, t);
        int acc = (dE <= 0) ? 1 : ((-dE * L.beta) > std::log(ev[i].u) ? 1 : 0);
        if (acc) L.spins[site] = t;
        if (acc_out) acc_out[i] = (uint8_t)acc;
        if (first_mismatch < 0 && acc != ev[i].accepted) first_mismatch = i;
    }
    return first_mismatch;
}

// Checkerboard Ising sweeps drawn from the same Philox counters as the GPU library, in FP32
// with the same operation order (dE = (H + sum_k J_k s_k) * (s - t); accept if dE <= 0 or
// -dE*beta > logf(u)). Used to show that the GPU Ising chain is the same chain, bit for bit.
void cb_ising(Lattice& L, uint64_t seed, uint32_t chain, uint64_t sweep0, int nsweeps,
              const float* Jdir, int ndir, const int (*dirs)[3], float Hx) {
    const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    const float beta = (float)L.beta;
    for (int sw = 0; sw < nsweeps; ++sw) {
        uint64_t s = sweep0 + (uint64_t)sw;
        for (int colour = 0; colour < 2; ++colour) {
            for (size_t i = 0; i < L.spins.size(); ++i) {
                const I4& l = L.locs[i];
                int par = (l[0] + l[1] + l[2]) & 1;
                if (par != colour) continue;
                uint32_t box = (uint32_t)L.box_index(l);
                uint32_t c[4] = {box, (uint32_t)s, (uint32_t)(s >> 32) | (STREAM_SWEEP << 28), chain};
                philox10(c, k0, k1);
                float t = (c[0] >> 31) ? 1.0f : -1.0f;
                float u = ((float)(c[1] >> 9) + 0.5f) * (1.0f / 8388608.0f);   // (0,1), exact
                float h = Hx;
                for (int k = 0; k < ndir; ++k) {
                    I4 q = l;
                    for (int a = 0; a < 3; ++a) q[a] += dirs[k][a];
                    bool ok = true;
                    for (int a = 0; a < L.d; ++a) {
                        if (L.periodic) q[a] = (q[a] + L.edge) % L.edge;
                        else if (q[a] < 0 || q[a] >= L.edge) ok = false;
                    }
                    float sn = 0.0f;
                    if (ok) {
                        int j = L.box_to_site[L.box_index(q)];
                        if (j >= 0) sn = (float)L.spins[j][0];
                    }
                    h = h + Jdir[k] * sn;
                }
                float so = (float)L.spins[i][0];
                float dE = h * (so - t);
                bool acc = (dE <= 0.0f) || (-dE * beta > logf(u));
                if (acc) L.spins[i][0] = t;
            }
        }
    }
}

// The colour-class order of libnmmc's general-table sweep for Ising chains: every sweep visits
// classes 0..q-1 (kind 1: (x + b*y + c*z) mod q; kind 2: x mod p + p*(y mod p) + p^2*(z mod p));
// no two sites of a class interact, so the order inside a class is immaterial. FP32 field over
// the interaction records in file order, one Philox draw per site as in cb_ising.
void colour_ising(Lattice& L, uint64_t seed, uint32_t chain, uint64_t sweep0, int nsweeps, int kind, int q,
                  int p, int b, int c, float Hx) {
    const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    const float beta = (float)L.beta;
    auto colour_of = [&](const I4& l) {
        if (kind == 1) return (int)((((long)l[0] + (long)b * l[1] + (long)c * l[2]) % q + q) % q);
        return (l[0] % p) + p * (l[1] % p) + p * p * (L.d == 3 ? l[2] % p : 0);
    };
    for (int sw = 0; sw < nsweeps; ++sw) {
        uint64_t s = sweep0 + (uint64_t)sw;
        for (int colour = 0; colour < q; ++colour) {
            for (size_t i = 0; i < L.spins.size(); ++i) {
                const I4& l = L.locs[i];
                if (colour_of(l) != colour) continue;
                uint32_t box = (uint32_t)L.box_index(l);
                uint32_t ctr[4] = {box, (uint32_t)s, (uint32_t)(s >> 32) | (STREAM_SWEEP << 28), chain};
                philox10(ctr, k0, k1);
                float t = (ctr[0] >> 31) ? 1.0f : -1.0f;
                float u = ((float)(ctr[1] >> 9) + 0.5f) * (1.0f / 8388608.0f);   // (0,1), exact
                float h = Hx;
                for (size_t j = 0; j < L.neigh[i].size(); ++j) {   // file order, as set_neigh
                    float J = L.useJ ? (float)L.J_diffs[L.neigh_choice[i][j]] : 0.0f;
                    h = h + J * (float)L.spins[L.neigh[i][j]][0];
                }
                float so = (float)L.spins[i][0];
                float dE = h * (so - t);
                bool acc = (dE <= 0.0f) || (-dE * beta > logf(u));
                if (acc) L.spins[i][0] = t;
            }
        }
    }
}

int read_interactions(const char* path, int d, double Jmod, double Dmod,
                      std::vector<I4>& offs, std::vector<double>& J, std::vector<V4>& D) {
    // field_type.cpp:39-73: d ints, then J, then 3 D components per record
    std::ifstream f(path);
    if (!f.is_open()) return -1;
    int icurr;
    double dcurr;
    while (f >> icurr) {
        I4 loc{0, 0, 0, 0};
        V4 dmi{0, 0, 0, 0};
        loc[0] = icurr;
        for (int i = 1; i < d; ++i) {
            f >> icurr;
            loc[i] = icurr;
        }
        offs.push_back(loc);
        f >> dcurr;
        J.push_back(Jmod * dcurr);
        for (int i = 0; i < 3; ++i) {
            f >> dcurr;
            dmi[i] = Dmod * dcurr;
        }
        D.push_back(dmi);
    }
    return (int)offs.size();
}

}  // namespace

// ========================================================================================
// C interface (ctypes)
// ========================================================================================
extern "C" {

void* orc_create(int d, int edge, int ising, int periodic, char shape, double size, double wbeta,
                 uint64_t seed, uint32_t chain, const uint8_t* mask_in,
                 int n_off, const int* offsets, const double* J, const double* D,
                 int useJ, int useD) {
    Lattice* L = new Lattice();
    L->d = d;
    L->edge = edge;
    L->ising = ising != 0;
    L->periodic = periodic != 0;
    L->shape = shape;
    L->wsize = size;
    L->wbeta = wbeta;
    if (wbeta > 0) L->wr0 = 1 / std::tgamma(1. + 1. / wbeta);   // shape.cpp:22
    L->useJ = useJ != 0;
    L->useD = useD != 0;
    set_default_spins(*L);
    for (int k = 0; k < n_off; ++k) {
        L->loc_diffs.push_back(I4{offsets[3 * k], offsets[3 * k + 1], d == 3 ? offsets[3 * k + 2] : 0, 0});
        L->J_diffs.push_back(J[k]);
        L->D_vecs.push_back(V4{D[3 * k], D[3 * k + 1], D[3 * k + 2], 0});
    }
    init_lattice(*L, mask_in, seed, chain);
    set_neigh(*L);
    return L;
}

// Test fixtures of Old/tests/test_functions.hpp: kind 0 = gen_fm, 1 = gen_afm, 2 = gen_skyrm.
void* orc_fixture(int kind, int d, int ising, int periodic, int n_off, const int* offsets,
                  const double* J, const double* D) {
    Lattice* L = new Lattice();
    int edge = (kind == 2) ? 30 : 10;
    L->d = d;
    L->edge = edge;
    L->ising = (kind == 2) ? false : (ising != 0);
    L->periodic = (kind == 0) ? (periodic != 0) : false;   // gen_afm / gen_skyrm: never periodic
    L->shape = (d == 3) ? 'c' : 's';
    set_default_spins(*L);
    for (int k = 0; k < n_off; ++k) {
        L->loc_diffs.push_back(I4{offsets[3 * k], offsets[3 * k + 1], d == 3 ? offsets[3 * k + 2] : 0, 0});
        L->J_diffs.push_back(J[k]);
        L->D_vecs.push_back(V4{D[3 * k], D[3 * k + 1], D[3 * k + 2], 0});
    }
    int pos[3] = {0, 0, 0};
    long total = 1;
    for (int k = 0; k < d; ++k) total *= edge;
    int mid = edge / 2;
    float sk_R = mid - 3;
    float kk = (float)M_PI / sk_R;
    for (long i = 0; i < total; ++i) {
        I4 loc{pos[0], pos[1], d == 3 ? pos[2] : 0, 0};
        add_spin(*L, loc);
        if (kind == 1) {
            int possum = 0;
            for (int j = 0; j < d; ++j) possum += pos[j];
            if (possum % 2 == 1) L->spins.back() = L->downspin;
        } else if (kind == 2) {
            float dx = pos[0] - mid, dy = pos[1] - mid;
            float r2 = (float)(std::pow(dx, 2) + std::pow(dy, 2));
            float r = (float)std::pow(r2, 0.5);
            V4 sp{0, 0, 0, 0};
            if (!(r >= sk_R)) {
                float phi = std::atan2(dx, dy);
                sp[0] = -std::sin(kk * r) * std::cos(phi);
                sp[1] = std::sin(kk * r) * std::sin(phi);
                sp[2] = std::cos(kk * r);
            }
            L->spins.back() = sp;
        }
        for (int j = d - 1; j >= 0; --j) {
            if (++pos[j] < edge) break;
            pos[j] = 0;
        }
    }
    set_neigh(*L);
    return L;
}

void orc_destroy(void* h) { delete (Lattice*)h; }
int orc_num_sites(void* h) { return (int)((Lattice*)h)->spins.size(); }
int orc_snum(void* h) { return ((Lattice*)h)->snum; }
int orc_s4num(void* h) { return ((Lattice*)h)->s4num; }
void orc_set_flags(void* h, int useJ, int useD, int dmi_sign) {
    Lattice* L = (Lattice*)h;
    L->useJ = useJ != 0;
    L->useD = useD != 0;
    L->dmi_sign = dmi_sign;
}
void orc_set_H(void* h, double hx, double hy, double hz) {
    Lattice* L = (Lattice*)h;
    L->H = {hx, hy, hz, 0};
}
void orc_set_beta(void* h, double beta) { ((Lattice*)h)->beta = beta; }
void orc_locs(void* h, int* out) {
    Lattice* L = (Lattice*)h;
    for (size_t i = 0; i < L->locs.size(); ++i)
        for (int c = 0; c < 3; ++c) out[3 * i + c] = L->locs[i][c];
}
void orc_get_spins(void* h, double* out) {
    Lattice* L = (Lattice*)h;
    for (size_t i = 0; i < L->spins.size(); ++i)
        for (int c = 0; c < 3; ++c) out[3 * i + c] = L->spins[i][c];
}
void orc_set_spins(void* h, const double* in) {
    Lattice* L = (Lattice*)h;
    for (size_t i = 0; i < L->spins.size(); ++i)
        for (int c = 0; c < 3; ++c) L->spins[i][c] = in[3 * i + c];
}
// Random start (field_type.cpp:197-204)
void orc_all_rand(void* h, void* rng) {
    Lattice* L = (Lattice*)h;
    for (size_t i = 0; i < L->spins.size(); ++i) {
        gen_rand(*L, *(RngSet*)rng);
        L->spins[i] = L->testspin;
    }
}
int orc_neighbours(void* h, int site, int* nb, int* choice, int cap) {
    Lattice* L = (Lattice*)h;
    int n = (int)L->neigh[site].size();
    for (int j = 0; j < n && j < cap; ++j) {
        nb[j] = L->neigh[site][j];
        choice[j] = L->neigh_choice[site][j];
    }
    return n;
}
void orc_adj(void* h, int* out) {
    Lattice* L = (Lattice*)h;
    for (size_t i = 0; i < L->adj.size(); ++i)
        for (int c = 0; c < 4; ++c) out[4 * i + c] = L->adj[i][c];
}

double orc_energy(void* h) { return calc_E(*(Lattice*)h); }
double orc_dE(void* h, int site, const double* trial) {
    V4 t{trial[0], trial[1], trial[2], 0};
    return calc_dE(*(Lattice*)h, site, t);
}
void orc_mag(void* h, double* out) {
    V4 m = calc_M(*(Lattice*)h);
    for (int c = 0; c < 3; ++c) out[c] = m[c];
}
void orc_submag(void* h, int sub, double* out) {
    V4 m = calc_subM(*(Lattice*)h, sub);
    for (int c = 0; c < 3; ++c) out[c] = m[c];
}
void orc_sub4mag(void* h, double* out) {
    V4 m = calc_sub4M(*(Lattice*)h);
    for (int c = 0; c < 3; ++c) out[c] = m[c];
}
int orc_tcharge(void* h, double* out) {
    std::vector<double> q = calc_TC(*(Lattice*)h);
    for (size_t i = 0; i < q.size(); ++i) out[i] = q[i];
    return (int)q.size();
}
double orc_solid_angle(const double* a, const double* b, const double* c) {
    V4 s1{a[0], a[1], a[2], 0}, s2{b[0], b[1], b[2], 0}, s3{c[0], c[1], c[2], 0};
    return solid_angle(s1, s2, s3);
}

void* orc_rng_create(unsigned long seed_int, unsigned long seed_double, unsigned long seed_sphere) {
    return new RngSet(seed_int, seed_double, seed_sphere);
}
void orc_rng_destroy(void* r) { delete (RngSet*)r; }
double orc_rng_uniform(void* r) { return ((RngSet*)r)->rdouble.uniform(); }
int orc_rng_int2(void* r) { return ((RngSet*)r)->rint.uniform_int2(); }
void orc_rng_dir3d(void* r, double* out) { ((RngSet*)r)->rsphere.dir3d(out[0], out[1], out[2]); }
double orc_rng_lognormal(void* r, double zeta, double sigma) { return ((RngSet*)r)->rdouble.lognormal(zeta, sigma); }
// Bulk draws for the distribution tests (Old/tests/rand_test.hpp): kind 0 uniform, 1 {0,1}
// integer, 2 log-normal(a, b), 3 direction on S^2 (3 doubles per draw), each from the
// generator the reference uses for that draw.
void orc_rng_fill(void* r, int kind, long n, double a, double b, double* out) {
    RngSet& g = *(RngSet*)r;
    for (long i = 0; i < n; ++i) {
        switch (kind) {
            case 0: out[i] = g.rdouble.uniform(); break;
            case 1: out[i] = g.rint.uniform_int2(); break;
            case 2: out[i] = g.rdouble.lognormal(a, b); break;
            default: g.rsphere.dir3d(out[3 * i], out[3 * i + 1], out[3 * i + 2]); break;
        }
    }
}
// testspin generation only (used by the dE-consistency tests, heis_test.hpp:344-376)
void orc_gen_rand(void* h, void* r, double* out) {
    Lattice* L = (Lattice*)h;
    gen_rand(*L, *(RngSet*)r);
    for (int c = 0; c < 3; ++c) out[c] = L->testspin[c];
}

void orc_equil(void* h, void* rng, long iter, void* event_log) {
    equil(*(Lattice*)h, *(RngSet*)rng, iter, (Event*)event_log);
}
long orc_replay(void* h, const void* events, long n, uint8_t* acc_out) {
    return replay(*(Lattice*)h, (const Event*)events, n, acc_out);
}
int orc_event_size(void) { return (int)sizeof(Event); }

void orc_cb_ising(void* h, uint64_t seed, uint32_t chain, uint64_t sweep0, int nsweeps,
                  const float* Jdir, int ndir, const int* dirs, float Hx) {
    cb_ising(*(Lattice*)h, seed, chain, sweep0, nsweeps, Jdir, ndir, (const int(*)[3])dirs, Hx);
}

void orc_colour_ising(void* h, uint64_t seed, uint32_t chain, uint64_t sweep0, int nsweeps, int kind, int q,
                      int p, int b, int c, float Hx) {
    colour_ising(*(Lattice*)h, seed, chain, sweep0, nsweeps, kind, q, p, b, c, Hx);
}

void orc_philox(const uint32_t* ctr, const uint32_t* key, uint32_t* out) {
    uint32_t c[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
    philox10(c, key[0], key[1]);
    for (int i = 0; i < 4; ++i) out[i] = c[i];
}
// The four sweep-stream words of boxes box0 .. box0+nbox-1 for one (seed, chain, sweep):
// counter {box, sweep lo, sweep hi | stream << 28, chain}, key {seed lo, seed hi}.
void orc_philox_boxes(uint64_t seed, uint32_t chain, uint64_t sweep, uint32_t stream, uint32_t box0,
                      long nbox, uint32_t* out) {
    for (long i = 0; i < nbox; ++i) {
        uint32_t c[4] = {box0 + (uint32_t)i, (uint32_t)sweep, (uint32_t)(sweep >> 32) | (stream << 28), chain};
        philox10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
        for (int k = 0; k < 4; ++k) out[4 * i + k] = c[k];
    }
}
double orc_mask_uniform(uint64_t seed, uint32_t chain, uint32_t box) { return mask_uniform(seed, chain, box); }

// Interaction file reader: returns the number of records, -1 if the file cannot be opened.
int orc_read_interactions(const char* path, int d, double Jmod, double Dmod, int cap,
                          int* offsets, double* J, double* D) {
    std::vector<I4> o;
    std::vector<double> j;
    std::vector<V4> dv;
    int n = read_interactions(path, d, Jmod, Dmod, o, j, dv);
    for (int k = 0; k < n && k < cap; ++k) {
        for (int c = 0; c < 3; ++c) offsets[3 * k + c] = o[k][c];
        J[k] = j[k];
        for (int c = 0; c < 3; ++c) D[3 * k + c] = dv[k][c];
    }
    return n;
}

// Timed random-site update loop for the CPU baseline: returns attempts performed.
long orc_bench_equil(void* h, void* rng, long iter) {
    equil(*(Lattice*)h, *(RngSet*)rng, iter, nullptr);
    return iter;
}

}  // extern "C"
