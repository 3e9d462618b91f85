// The learned warm start's 3-sigma gate and random-start fallback for C and C++ callers, on
// top of the public C ABI (no reference counterpart: the reference always starts from random
// spins, Old/lib/field_type.cpp:197-204).
//
// A warm start is kept only if the plain Metropolis chain, run from it, gives E/N, |M|/N and
// Q that agree within 3 standard errors with a reference: either statistics of long plain
// chains (nmmc_reference_stats) or, without one, the same chains' next window of samples (a
// drift test). Otherwise the chains are restarted from uniform random spins.
#include <math.h>
#include <string.h>

#include <vector>

#include "../../include/nmmc.h"

namespace {

// Per observable (E/N, |M|/N, Q): the grand mean over samples and chains, the spread of one
// chain's instantaneous value, and the standard error of the mean from the per-chain averages
// (independent chains, so each chain's autocorrelation is absorbed).
void window_stats(const double* obs, int nsamp, int n, const std::vector<double>& sites, double out[9]) {
    static const int idx[3] = {NMMC_OBS_E, NMMC_OBS_ABSM, NMMC_OBS_QTOT};
    for (int o = 0; o < 3; ++o) {
        double sum = 0, sum2 = 0;
        std::vector<double> cm(n, 0.0);
        for (int s = 0; s < nsamp; ++s)
            for (int i = 0; i < n; ++i) {
                double v = obs[((size_t)s * n + i) * NMMC_OBS_N + idx[o]];
                if (o < 2) v /= sites[i];
                sum += v;
                sum2 += v * v;
                cm[i] += v / nsamp;
            }
        const double cnt = (double)nsamp * n;
        const double mean = sum / cnt;
        const double sd = cnt > 1 ? sqrt(fmax(0.0, (sum2 - cnt * mean * mean) / (cnt - 1))) : 0.0;
        double m = 0, v2 = 0;
        for (double c : cm) m += c / n;
        for (double c : cm) v2 += (c - m) * (c - m);
        const double se = n > 1 ? sqrt(v2 / (n - 1) / n) : INFINITY;
        out[3 * o] = mean;
        out[3 * o + 1] = sd;
        out[3 * o + 2] = se;
    }
}

int filled_sites(nmmc_ctx* ctx, const int* chains, int n, std::vector<double>& sites) {
    sites.resize(n);
    for (int i = 0; i < n; ++i) {
        int num = 0;
        if (int rc = nmmc_site_counts(ctx, chains[i], &num, nullptr, nullptr)) return rc;
        sites[i] = num > 0 ? num : 1;
    }
    return NMMC_OK;
}

// One 64-bit mixing step (splitmix64) for the fallback's random spins.
uint64_t mix(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

}  // namespace

extern "C" int nmmc_reference_stats(nmmc_ctx* ctx, const int* chains, int n, int eq_sweeps, int nsamp, int gap,
                                    double out[9]) {
    if (!ctx || !chains || !out || n <= 0 || nsamp <= 0 || gap <= 0 || eq_sweeps < 0) return NMMC_ERR_ARG;
    std::vector<double> sites;
    int rc = filled_sites(ctx, chains, n, sites);
    if (rc) return rc;
    if ((rc = nmmc_sweep(ctx, chains, n, eq_sweeps))) return rc;
    std::vector<double> obs((size_t)nsamp * n * NMMC_OBS_N);
    if ((rc = nmmc_sample(ctx, chains, n, gap, nsamp, obs.data(), nullptr))) return rc;
    window_stats(obs.data(), nsamp, n, sites, out);
    return NMMC_OK;
}

extern "C" int nmmc_gen_gated_warm_start(nmmc_gen* gen, nmmc_ctx* ctx, const int* chains, int n, const double* cond,
                                         int steps, int check_sweeps, int nsamp, int gap, const double* ref,
                                         uint64_t seed, int* kept) {
    if (!gen || !ctx || !chains || !cond || !kept || n <= 0 || nsamp <= 0 || gap <= 0 || check_sweeps < 0)
        return NMMC_ERR_ARG;
    *kept = 0;
    std::vector<double> sites;
    int rc = filled_sites(ctx, chains, n, sites);
    if (rc) return rc;
    if ((rc = nmmc_gen_warm_start(gen, ctx, chains, n, cond, steps, 2))) return rc;
    if ((rc = nmmc_sweep(ctx, chains, n, check_sweeps))) return rc;
    std::vector<double> obs((size_t)nsamp * n * NMMC_OBS_N);
    if ((rc = nmmc_sample(ctx, chains, n, gap, nsamp, obs.data(), nullptr))) return rc;
    double got[9], against[9];
    window_stats(obs.data(), nsamp, n, sites, got);
    if (ref) {
        memcpy(against, ref, sizeof(against));
    } else {   // drift test: the next window of the same chains
        if ((rc = nmmc_sample(ctx, chains, n, gap, nsamp, obs.data(), nullptr))) return rc;
        window_stats(obs.data(), nsamp, n, sites, against);
    }
    int keep = 1;
    for (int o = 0; o < 3; ++o) {
        const double d = fabs(got[3 * o] - against[3 * o]);
        const double se = hypot(got[3 * o + 2], against[3 * o + 2]);
        if (!(d <= 3.0 * se + 1e-12)) keep = 0;
    }
    if (!keep) {   // the reference's start: uniform random spins (Old/lib/field_type.cpp:197-204)
        nmmc_info info;
        if ((rc = nmmc_get_info(ctx, &info))) return rc;
        std::vector<double> xyz((size_t)info.box_sites * 3);
        std::vector<uint8_t> mask((size_t)info.box_sites);
        uint64_t st = seed ^ 0xA0761D6478BD642Full;
        for (int i = 0; i < n; ++i) {
            if ((rc = nmmc_get_mask(ctx, chains[i], mask.data(), (size_t)info.box_sites))) return rc;
            for (long long b = 0; b < info.box_sites; ++b) {
                double* v = &xyz[3 * (size_t)b];
                if (!mask[b]) {
                    v[0] = v[1] = v[2] = 0.0;
                    continue;
                }
                // Archimedes: z uniform in [-1, 1), azimuth uniform
                const double u1 = (double)(mix(st) >> 11) * 0x1.0p-53, u2 = (double)(mix(st) >> 11) * 0x1.0p-53;
                const double z = 2.0 * u1 - 1.0, ph = 2.0 * M_PI * u2, r = sqrt(fmax(0.0, 1.0 - z * z));
                v[0] = r * cos(ph);
                v[1] = r * sin(ph);
                v[2] = z;
            }
            if ((rc = nmmc_set_spins(ctx, chains[i], xyz.data(), (size_t)info.box_sites))) return rc;
        }
    }
    *kept = keep;
    return NMMC_OK;
}
