// Host-side part of libnmmc: input-file reader, list loader, interaction reader, protocol
// plan, particle sizes and shapes, binning statistics. Plain C++17; no CUDA.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <array>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "nmmc_hostlib.h"
#include "philox.h"

namespace nmmc {

namespace {
thread_local std::string g_err;
}

int set_error_host(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

int set_error(int code, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

// ------------------------------------------------------------------------------------------
// read_var (Old/lib/param_read.cpp:8-33): the first line whose first token is the key wins;
// the value is the next token, converted like `stream >> value`.
// ------------------------------------------------------------------------------------------
namespace {

struct InputFile {
    std::vector<std::string> lines;
    bool ok = false;
};

InputFile load_file(const char* path) {
    InputFile f;
    std::ifstream in(path);
    if (!in.is_open()) return f;
    std::string line;
    while (std::getline(in, line)) f.lines.push_back(line);
    f.ok = true;
    return f;
}

template <class T>
bool read_var(const InputFile& f, const char* key, T& out) {
    for (const std::string& line : f.lines) {
        std::istringstream s(line);
        std::string name;
        T v{};
        s >> name >> v;
        if (name == key) {
            out = v;
            return true;
        }
    }
    return false;
}

}  // namespace

double derived_edge(char shape, double amean, double asd) {
    switch (shape) {
        case 'w': case 'W': case 'x': case 'X': return (amean + 2 * asd) * 3;
        case 's': case 'S': case 'c': case 'C': return amean + 2 * asd;
        default: return 0;
    }
}

int shape_dim(char shape) {
    switch (shape) {
        case 's': case 'S': case 'w': case 'W': return 2;
        case 'c': case 'C': case 'x': case 'X': return 3;
        default: return 0;
    }
}

bool shape_is_weibull(char shape) {
    return shape == 'w' || shape == 'W' || shape == 'x' || shape == 'X';
}

// A record couples two sites when its J or (Heisenberg) D is nonzero.
static bool record_couples(const nmmc_interactions& in, int r, bool ising) {
    if (in.J[r] != 0) return true;
    if (!ising)
        for (int c = 0; c < 3; ++c)
            if (in.D[r][c] != 0) return true;
    return false;
}

int map_interactions(const nmmc_interactions& in, int dim, bool ising, double J[6], double D[6][3],
                     bool& general, std::string& why) {
    for (int k = 0; k < 6; ++k) {
        J[k] = 0;
        D[k][0] = D[k][1] = D[k][2] = 0;
    }
    general = false;
    for (int r = 0; r < in.n; ++r) {
        const int* o = in.offset[r];
        for (int a = dim; a < 3; ++a)
            if (o[a] != 0) {
                why = "interaction offset uses an axis the lattice does not have";
                return NMMC_ERR_UNSUPPORTED;
            }
        int nz = 0, axis = -1, sign = 0;
        for (int a = 0; a < dim; ++a)
            if (o[a] != 0) {
                nz++;
                axis = a;
                sign = o[a];
            }
        if (nz == 0) continue;   // self-offset: the reference skips i == j
        if (nz != 1 || (sign != 1 && sign != -1)) {
            if (record_couples(in, r, ising)) general = true;
            continue;
        }
        int dir = 2 * axis + (sign > 0 ? 0 : 1);
        J[dir] += in.J[r];
        for (int c = 0; c < 3; ++c) D[dir][c] += in.D[r][c];
    }
    if (general)
        for (int k = 0; k < 6; ++k) {
            J[k] = 0;
            D[k][0] = D[k][1] = D[k][2] = 0;
        }
    return NMMC_OK;
}

int find_colouring(const nmmc_interactions& in, int dim, int edge, bool periodic, bool ising, Colouring& out,
                   std::string& why) {
    // coupling offsets, reduced to the symmetric residue on a periodic lattice; self-offsets
    // (after the wrap) are skipped by the sweep, as the reference skips i == j
    std::vector<std::array<int, 3>> offs;
    int R = 0;
    for (int r = 0; r < in.n; ++r) {
        if (!record_couples(in, r, ising)) continue;
        std::array<int, 3> o{0, 0, 0};
        bool self = true;
        for (int a = 0; a < dim; ++a) {
            int v = in.offset[r][a];
            if (periodic) {
                v = ((v % edge) + edge) % edge;
                if (v > edge / 2) v -= edge;
            }
            o[a] = v;
            if (v != 0) self = false;
            R = std::max(R, std::abs(v));
        }
        if (!self) offs.push_back(o);
    }
    std::sort(offs.begin(), offs.end());
    offs.erase(std::unique(offs.begin(), offs.end()), offs.end());
    auto fits = [&](int period) { return !periodic || edge % period == 0; };
    // linear colourings, fewest colours first
    const int qmax = std::min(dim == 3 ? 48 : 128, std::max(2, edge));
    for (int q = 2; q <= qmax; ++q) {
        if (!fits(q)) continue;
        for (int b = 0; b < q; ++b)
            for (int c = 0; c < (dim == 3 ? q : 1); ++c) {
                bool ok = true;
                for (const auto& o : offs) {
                    long v = ((long)o[0] + (long)b * o[1] + (long)c * o[2]) % q;
                    if (v == 0) {
                        ok = false;
                        break;
                    }
                }
                if (ok) {
                    out.kind = 1;
                    out.q = out.p = q;
                    out.b = b;
                    out.c = c;
                    return NMMC_OK;
                }
            }
    }
    // product colouring: period p > R on every axis
    for (int p = std::max(2, R + 1); p <= edge; ++p) {
        if (!fits(p)) continue;
        long q = 1;
        for (int a = 0; a < dim; ++a) q *= p;
        if (q > 4096) break;
        out.kind = 2;
        out.p = p;
        out.q = (int)q;
        out.b = out.c = 0;
        return NMMC_OK;
    }
    char msg[200];
    snprintf(msg, sizeof msg,
             "no parallel colouring of %d colours or fewer for this interaction table (reach %d, edge %d%s)",
             4096, R, edge, periodic ? ", periodic" : "");
    why = msg;
    return NMMC_ERR_UNSUPPORTED;
}

void weibull_mask(int dim, int edge, double a, double wbeta, uint64_t seed, uint32_t chain,
                  uint8_t* mask) {
    const double r0 = 1 / tgamma(1. + 1. / wbeta);   // Old/lib/shape.cpp:22
    const double centre = double(edge - 1) / 2.;
    const int nz = (dim == 3) ? edge : 1;
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < edge; ++y)
            for (int x = 0; x < edge; ++x) {
                int pos[3] = {x, y, z};
                double dist2 = 0;
                for (int i = 0; i < dim; ++i) dist2 += pow((pos[i] - centre) / a, 2);
                double dist = pow(dist2, 0.5);
                double test = exp(-pow((dist / r0), wbeta));
                uint32_t box = (uint32_t)(x + edge * (y + edge * z));
                nmmc_u4 r = nmmc_philox(box, 0u, NMMC_STREAM_MASK << 28, chain, (uint32_t)seed,
                                        (uint32_t)(seed >> 32));
                mask[box] = (nmmc_u01d(r.x) < test) ? 1 : 0;
            }
}

void site_counts(int dim, int edge, const uint8_t* mask, int* num, int* snum, int* s4num) {
    int n = 0, s = 0, s4 = 0;
    const int nz = (dim == 3) ? edge : 1;
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < edge; ++y)
            for (int x = 0; x < edge; ++x) {
                long box = x + (long)edge * (y + (long)edge * z);
                if (mask && !mask[box]) continue;
                n++;
                if ((x + y + z) % 2 == 0) s++;
                int possum2 = x + y;
                int posdiff = -x + y + (edge - edge % 4);
                if (possum2 % 4 == 0 && posdiff % 4 == 0 && z % 4 == 0) s4++;
                else if (possum2 % 4 == 2 && posdiff % 4 == 2 && z % 4 == 2) s4++;
            }
    *num = n;
    *snum = s;
    *s4num = s4;
}

}  // namespace nmmc

using namespace nmmc;

extern "C" {

const char* nmmc_last_error(void) { return g_err.c_str(); }

int nmmc_read_input(const char* path, nmmc_options* o) {
    if (!path || !o) return set_error(NMMC_ERR_ARG, "null argument");
    InputFile f = load_file(path);
    if (!f.ok) return set_error(NMMC_ERR_INPUT, "Input file not opened: %s", path);
    memset(o, 0, sizeof *o);
    auto need = [&](auto& dst, const char* key) -> bool {
        if (read_var(f, key, dst)) return true;
        set_error(NMMC_ERR_INPUT, "Variable name '%s' not found", key);
        return false;
    };
    std::string s;
    int iv = 0;
    double dv = 0;
    char cv = 0;
    // Old/lib/param_read.cpp:37-81, in the same order (the first missing key is reported).
    if (!need(iv, "ISISING")) return NMMC_ERR_INPUT;
    o->is_ising = iv;
    if (!need(dv, "EXCHANGE")) return NMMC_ERR_INPUT;
    o->J = dv;
    if (!need(dv, "DMISTREN")) return NMMC_ERR_INPUT;
    o->K = dv;
    if (!need(iv, "ISDISTRIB")) return NMMC_ERR_INPUT;
    o->distrib = iv;
    if (o->distrib) {
        if (!need(dv, "MEANSIZE")) return NMMC_ERR_INPUT;
        o->amean = dv;
        if (!need(dv, "SIZEDEV")) return NMMC_ERR_INPUT;
        o->asd = dv;
    } else {
        if (!need(dv, "SIZE")) return NMMC_ERR_INPUT;
        o->amean = dv;
        o->asd = 0;
    }
    if (!need(cv, "LATTSHAPE")) return NMMC_ERR_INPUT;
    o->shape_code = cv;
    if (shape_is_weibull(cv)) {
        if (!need(dv, "WEIBULLFACT")) return NMMC_ERR_INPUT;
        o->beta_w = dv;
    }
    o->edge_size = derived_edge(cv, o->amean, o->asd);
    if (!need(iv, "NLATTS")) return NMMC_ERR_INPUT;
    o->n_latts = iv;
    if (!need(dv, "BOLTZMANN")) return NMMC_ERR_INPUT;
    o->k_b = dv;
    if (!need(iv, "ISPERIO")) return NMMC_ERR_INPUT;
    o->is_perio = iv;
    if (!need(iv, "SAMPSWEEPS")) return NMMC_ERR_INPUT;
    o->samp_sweeps = iv;
    if (!need(iv, "EQSWEEPS")) return NMMC_ERR_INPUT;
    o->eq_sweeps = iv;
    if (!need(iv, "NSAMPS")) return NMMC_ERR_INPUT;
    o->n_samp = iv;
    if (!need(s, "TEMPNAME")) return NMMC_ERR_INPUT;
    snprintf(o->temp_file, NMMC_MAX_PATH, "%s", s.c_str());
    if (!need(s, "FIELDNAME")) return NMMC_ERR_INPUT;
    snprintf(o->field_file, NMMC_MAX_PATH, "%s", s.c_str());
    if (!need(iv, "PROTOCOL")) return NMMC_ERR_INPUT;
    o->protocol = iv;
    if (!need(s, "INTERACTIONS")) return NMMC_ERR_INPUT;
    snprintf(o->int_file, NMMC_MAX_PATH, "%s", s.c_str());
    // Not read by the reference: the output name (main.cpp passes simOpt.outFile through).
    if (read_var(f, "OUTFILE", s)) snprintf(o->out_file, NMMC_MAX_PATH, "%s", s.c_str());
    o->size = o->amean;
    o->H = 0;       // the reference never sets stateOptions.H before the first state
    o->T = 1;
    if (o->distrib && o->amean > 0) {   // AtoLn, Old/lib/functions.cpp:56-62
        double av = pow(o->asd, 2), am2 = pow(o->amean, 2);
        o->lmean = log(am2 / pow(av + am2, 0.5));
        o->lsd = pow(log(1 + av / am2), 0.5);
    }
    return NMMC_OK;
}

static int load_list(const std::string& path, double* out, int cap, int* n) {
    std::ifstream f(path);
    if (!f.is_open()) return set_error(NMMC_ERR_INPUT, "list file not opened: %s", path.c_str());
    double v;
    int k = 0;
    while (f >> v) {
        if (k < cap && out) out[k] = (double)(float)v;   // stored as float (param_read.cpp:110)
        k++;
    }
    *n = k;
    if (k == 0) return set_error(NMMC_ERR_INPUT, "list file is empty: %s", path.c_str());
    return NMMC_OK;
}

int nmmc_load_lists(const nmmc_options* opt, const char* dir, double* Ts, int cap_T, int* n_T,
                    double* Hs, int cap_H, int* n_H) {
    if (!opt || !n_T || !n_H) return set_error(NMMC_ERR_ARG, "null argument");
    std::string base = dir ? std::string(dir) : std::string(".");
    if (!base.empty() && base.back() != '/') base += '/';
    int rc = load_list(base + "Temps/" + opt->temp_file, Ts, cap_T, n_T);
    if (rc) return rc;
    return load_list(base + "Fields/" + opt->field_file, Hs, cap_H, n_H);
}

int nmmc_colouring(int dim, int edge, int is_perio, int is_ising, const nmmc_interactions* inter, int out[5]) {
    if (!inter || !out || (dim != 2 && dim != 3) || edge < 1) return set_error(NMMC_ERR_ARG, "bad argument");
    double J[6], D[6][3];
    bool general = false;
    std::string why;
    int rc = map_interactions(*inter, dim, is_ising != 0, J, D, general, why);
    if (rc) return set_error_host(rc, why);
    Colouring col;
    if (general && (rc = find_colouring(*inter, dim, edge, is_perio != 0, is_ising != 0, col, why)))
        return set_error_host(rc, why);
    out[0] = col.kind;
    out[1] = col.q;
    out[2] = col.p;
    out[3] = col.b;
    out[4] = col.c;
    return NMMC_OK;
}

int nmmc_read_interactions(const char* path, int dim, double J_mod, double D_mod,
                           nmmc_interactions* out) {
    if (!path || !out) return set_error(NMMC_ERR_ARG, "null argument");
    std::ifstream f(path);
    if (!f.is_open()) return set_error(NMMC_ERR_INPUT, "interaction file not opened: %s", path);
    memset(out, 0, sizeof *out);
    out->dim = dim;
    int icurr;
    double dcurr;
    // Old/lib/field_type.cpp:49-71: dim ints, J, then three D components per record.
    while (f >> icurr) {
        if (out->n >= NMMC_MAX_OFFSETS)
            return set_error(NMMC_ERR_UNSUPPORTED, "more than %d interaction records in %s",
                             NMMC_MAX_OFFSETS, path);
        int r = out->n;
        out->offset[r][0] = icurr;
        for (int i = 1; i < dim; ++i) {
            f >> icurr;
            out->offset[r][i] = icurr;
        }
        f >> dcurr;
        out->J[r] = J_mod * dcurr;
        for (int i = 0; i < 3; ++i) {
            f >> dcurr;
            out->D[r][i] = D_mod * dcurr;
        }
        out->n++;
    }
    return NMMC_OK;
}

int nmmc_protocol_plan(int protocol, int n_H, int n_T, int* v1_is_T, int* v1_begin, int* v1_end,
                       int* v1_step, int* v2_begin, int* v2_end, int* v2_step) {
    // set_protocol / incr_v1 / incr_v2 (Old/lib/protocol.cpp:6-95)
    switch (protocol) {
        case 1:
            *v1_is_T = 0; *v1_begin = 0; *v1_end = n_H; *v1_step = 1;
            *v2_begin = 0; *v2_end = n_T; *v2_step = 1;
            return NMMC_OK;
        case 2:
            *v1_is_T = 1; *v1_begin = 0; *v1_end = n_T; *v1_step = 1;
            *v2_begin = 0; *v2_end = n_H; *v2_step = 1;
            return NMMC_OK;
        case 4:
            *v1_is_T = 1; *v1_begin = 0; *v1_end = n_T; *v1_step = 1;
            *v2_begin = n_H - 1; *v2_end = -1; *v2_step = -1;
            return NMMC_OK;
        default:
            return set_error(NMMC_ERR_PROTOCOL, "Invalid protocol %d", protocol);
    }
}

double nmmc_lognormal_size(uint64_t seed, int k, double lmean, double lsd) {
    nmmc_u4 r = nmmc_philox((uint32_t)k, 0u, NMMC_STREAM_SIZE << 28, 0u, (uint32_t)seed,
                            (uint32_t)(seed >> 32));
    double u1 = ((double)r.x + 0.5) * (1.0 / 4294967296.0);
    double u2 = ((double)r.y + 0.5) * (1.0 / 4294967296.0);
    double n = sqrt(-2.0 * log(u1)) * cos(2.0 * M_PI * u2);   // Box-Muller
    return exp(lmean + lsd * n);
}

int nmmc_shape_mask(char shape, int edge, double size, double wbeta, uint64_t seed, int lattice,
                    uint8_t* mask, int* num, int* snum, int* s4num) {
    const int dim = shape_dim(shape);
    if (!dim) return set_error(NMMC_ERR_SHAPE, "Incorrect shape code '%c'", shape);
    if (edge < 1 || !mask) return set_error(NMMC_ERR_ARG, "bad argument");
    long box = 1;
    for (int k = 0; k < dim; ++k) box *= edge;
    if (shape_is_weibull(shape)) {
        if (!(wbeta > 0)) return set_error(NMMC_ERR_ARG, "WEIBULLFACT must be positive");
        weibull_mask(dim, edge, size, wbeta, seed, (uint32_t)lattice, mask);
    } else {
        memset(mask, 1, (size_t)box);
    }
    int n, s, s4;
    site_counts(dim, edge, mask, &n, &s, &s4);
    if (num) *num = n;
    if (snum) *snum = s;
    if (s4num) *s4num = s4;
    return NMMC_OK;
}

int nmmc_binning(const double* x, int n, double* mean, double* err, double* tau) {
    if (!x || n < 2) return set_error(NMMC_ERR_ARG, "binning needs at least 2 samples");
    std::vector<double> b(x, x + n);
    double m = 0;
    for (double v : b) m += v;
    m /= n;
    auto level_err = [&](const std::vector<double>& v) {
        double mm = 0, s = 0;
        for (double t : v) mm += t;
        mm /= v.size();
        for (double t : v) s += (t - mm) * (t - mm);
        return sqrt(s / ((double)v.size() * (double)(v.size() - 1)));
    };
    double e0 = level_err(b), best = e0;
    // halve the series until fewer than 32 bins remain; the plateau estimate is the largest
    // error seen at a level that still has >= 32 bins
    while (b.size() >= 64) {
        std::vector<double> nb(b.size() / 2);
        for (size_t i = 0; i < nb.size(); ++i) nb[i] = 0.5 * (b[2 * i] + b[2 * i + 1]);
        b.swap(nb);
        best = std::max(best, level_err(b));
    }
    *mean = m;
    *err = best;
    if (tau) *tau = (e0 > 0) ? 0.5 * (best * best) / (e0 * e0) : 0.5;
    return NMMC_OK;
}

}  // extern "C"
