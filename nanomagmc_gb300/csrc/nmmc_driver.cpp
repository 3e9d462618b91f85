// Protocol driver: the program of Old/lib/main.cpp:18-309 on one GPU.
//
// Where the reference splits lattices and outer-protocol values over MPI ranks and hands the
// base state from rank to rank (main.cpp:104-275, protocol.cpp:97-131), this driver keeps
// every chain of the run in one context:
//   * one base chain per lattice, carried through v1 exactly like `base_state`
//     (initial 20*EQSWEEPS sweeps at Tmax, then EQSWEEPS per v1 value);
//   * at each v1 value the base chain is forked (curr_state = base_state, main.cpp:164)
//     into one inner chain per (v1, lattice);
//   * all inner chains then walk v2 together: EQSWEEPS per point, then NSAMPS samples
//     SAMPSWEEPS apart, each sample = energy, magnetisation, submag(0), sub4mag, tcharge.
// Sample arrays are written as .npy files with the shapes of Old/lib/output.cpp:161-249, and
// (unless ISDISTRIB) the summed and final lattices of lattice 0 at every point as
// Av_Latt/T_<t>-H_<h>.npy and Sing_Latt/T_<t>-H_<h>.npy (output.cpp:100-150);
// outdir/complete.npy holds the /Complete flags [v1, lattice] (output.cpp:429-444) and
// finished (v1, lattice) pairs are skipped on a rerun (main.cpp:167).
#include <math.h>
#include <stdio.h>
#include <string.h>
#include <sys/stat.h>

#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/nmmc.h"

namespace {

std::string join(const std::string& a, const std::string& b) {
    if (a.empty()) return b;
    if (!b.empty() && b[0] == '/') return b;
    return a.back() == '/' ? a + b : a + "/" + b;
}

// Minimal .npy (format 1.0) reader/writer for little-endian float32 / int32 C-order arrays.
bool write_npy(const std::string& path, const char* descr, const std::vector<long>& shape,
               const void* data, size_t elem) {
    std::string shp = "(";
    size_t n = 1;
    for (size_t i = 0; i < shape.size(); ++i) {
        shp += std::to_string(shape[i]);
        shp += (shape.size() == 1 || i + 1 < shape.size()) ? "," : "";
        if (i + 1 < shape.size()) shp += " ";
        n *= (size_t)shape[i];
    }
    shp += ")";
    std::string hdr = std::string("{'descr': '") + descr + "', 'fortran_order': False, 'shape': " + shp + ", }";
    size_t total = 10 + hdr.size() + 1;
    size_t pad = (64 - total % 64) % 64;
    hdr += std::string(pad, ' ') + "\n";
    std::string tmp = path + ".tmp";
    std::ofstream f(tmp, std::ios::binary);
    if (!f) return false;
    const char magic[] = "\x93NUMPY";
    f.write(magic, 6);
    char ver[2] = {1, 0};
    f.write(ver, 2);
    uint16_t hl = (uint16_t)hdr.size();
    f.write((const char*)&hl, 2);
    f.write(hdr.data(), hdr.size());
    f.write((const char*)data, n * elem);
    f.close();
    if (!f) return false;
    return rename(tmp.c_str(), path.c_str()) == 0;
}

// Reads a format-1.0 .npy file into data only if its dtype and shape are the expected ones
// (a file from a run with other sizes is ignored, not misread); false otherwise.
bool read_npy(const std::string& path, const char* descr, const std::vector<long>& shape, void* data,
              size_t bytes) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    char head[10];
    f.read(head, 10);
    if (!f || memcmp(head, "\x93NUMPY", 6) != 0 || head[6] != 1) return false;
    uint16_t hl;
    memcpy(&hl, head + 8, 2);
    std::string hdr(hl, '\0');
    f.read(&hdr[0], hl);
    if (!f) return false;
    auto field = [&](const char* key) -> std::string {   // text after 'key': up to the next , or )
        const size_t k = hdr.find(key);
        if (k == std::string::npos) return "";
        const size_t b = k + strlen(key);
        const size_t e = (hdr[b] == '(') ? hdr.find(')', b) + 1 : hdr.find(',', b);
        return (e == std::string::npos || e < b) ? "" : hdr.substr(b, e - b);
    };
    if (field("'descr': ") != std::string("'") + descr + "'") return false;
    if (field("'fortran_order': ") != "False") return false;
    std::vector<long> got;
    const std::string shp = field("'shape': ");
    for (size_t i = 0; i < shp.size();) {
        if (shp[i] >= '0' && shp[i] <= '9') {
            size_t j = i;
            while (j < shp.size() && shp[j] >= '0' && shp[j] <= '9') ++j;
            got.push_back(std::stol(shp.substr(i, j - i)));
            i = j;
        } else {
            ++i;
        }
    }
    if (got != shape) return false;
    std::vector<char> buf(bytes);
    f.read(buf.data(), (std::streamsize)bytes);
    if ((size_t)f.gcount() != bytes) return false;
    memcpy(data, buf.data(), bytes);
    return true;
}

// Keys nmmc_run reads beyond the reference's (whose reader ignores lines it does not look
// for): "GENERATOR <file>", a generator saved by nmmc_gen_save, relative to the work directory,
// "WSSTEPS <n>", its denoising passes (default 32), and "WSSCHED <k>", their noise levels
// (NMMC_GEN_OPT_SCHEDULE: 0 linear, 1 quadratic, 2 cosine; default 0). False when the file
// cannot be read or a value is out of range.
bool extra_keys(const char* input_path, std::string* genfile, int* ws_steps, int* ws_sched) {
    std::ifstream f(input_path);
    if (!f) return false;
    std::string key, line;
    while (std::getline(f, line)) {
        std::istringstream ls(line);
        if (!(ls >> key)) continue;
        if (key == "GENERATOR") ls >> *genfile;
        else if (key == "WSSTEPS") ls >> *ws_steps;
        else if (key == "WSSCHED") ls >> *ws_sched;
    }
    return *ws_steps > 0 && *ws_sched >= 0 && *ws_sched <= 2;
}

// The base chains' learned warm start at (Tmax, field 0, DMISTREN) behind the drift gate of
// nmmc_gen_gated_warm_start (EQSWEEPS check sweeps, then two windows of 20 samples 2 sweeps
// apart): kept, the chains skip the initial 20 * EQSWEEPS; rejected, they are back at random
// spins and take them as the reference does.
int warm_start_base(nmmc_ctx* ctx, const std::string& path, int edge, const std::vector<int>& base, double Tmax,
                    const nmmc_options& opt, int ws_steps, int ws_sched, uint64_t seed, int* kept) {
    nmmc_gen* gen = nullptr;
    int rc = nmmc_gen_create(edge, 0, seed ^ 0x9E3779B97F4A7C15ull, &gen);
    if (rc) return rc;
    rc = nmmc_gen_load(gen, path.c_str());
    if (!rc) rc = nmmc_gen_set_option(gen, NMMC_GEN_OPT_SCHEDULE, ws_sched);
    const int n = (int)base.size();
    std::vector<double> cond(3 * (size_t)n);
    for (int k = 0; k < n; ++k) {
        cond[3 * k] = Tmax;
        cond[3 * k + 1] = 0.0;   // the field before the first change_v1
        cond[3 * k + 2] = opt.K;
    }
    if (!rc)
        rc = nmmc_gen_gated_warm_start(gen, ctx, base.data(), n, cond.data(), ws_steps, opt.eq_sweeps, 20, 2, nullptr,
                                       seed, kept);
    nmmc_gen_destroy(gen);
    return rc;
}

}  // namespace

extern "C" int nmmc_run(const char* input_path, const char* workdir, const char* outdir, uint64_t seed,
                        int verbose) {
    if (!input_path || !outdir) return 300;
    const std::string wd = workdir ? workdir : ".";
    nmmc_options opt;
    int rc = nmmc_read_input(input_path, &opt);
    if (rc) return rc;
    const int dim = (opt.shape_code == 'c' || opt.shape_code == 'C' || opt.shape_code == 'x' || opt.shape_code == 'X') ? 3 : 2;
    std::vector<double> Ts(4096), Hs(4096);
    int nT = 0, nH = 0;
    if ((rc = nmmc_load_lists(&opt, wd.c_str(), Ts.data(), 4096, &nT, Hs.data(), 4096, &nH))) return rc;
    if (nT > 4096 || nH > 4096) return 300;
    Ts.resize(nT);
    Hs.resize(nH);
    nmmc_interactions inter;
    if ((rc = nmmc_read_interactions(join(join(wd, "Js"), opt.int_file).c_str(), dim, opt.J, opt.K, &inter))) return rc;
    int v1T, b1, e1, s1, b2, e2, s2;
    if ((rc = nmmc_protocol_plan(opt.protocol, nH, nT, &v1T, &b1, &e1, &s1, &b2, &e2, &s2))) return rc;
    const std::vector<double>& v1 = v1T ? Ts : Hs;
    const std::vector<double>& v2 = v1T ? Hs : Ts;
    const int nv1 = (int)v1.size();
    const int NL = opt.n_latts;
    if (NL <= 0) return 300;
    const double Tmax = Ts[0];   // main.cpp:46: lists are expected in descending order

    // chains: base chain k, then inner chain (i, k) at NL + i*NL + k
    std::vector<nmmc_chain_desc> ch((size_t)NL * (nv1 + 1));
    for (int k = 0; k < NL; ++k) {
        double size = opt.distrib ? nmmc_lognormal_size(seed, k, opt.lmean, opt.lsd) : opt.amean;
        for (int i = -1; i < nv1; ++i) {
            nmmc_chain_desc& d = ch[(size_t)NL + (size_t)i * NL + k];
            d.lattice = k;
            d.size = size;
            d.T = Tmax;
            d.H = 0.0;   // the reference leaves stateOptions.H unset before change_v1
        }
    }
    nmmc_ctx* ctx = nullptr;
    if ((rc = nmmc_create(&opt, &inter, ch.data(), (int)ch.size(), seed, &ctx))) return rc;
    nmmc_info info;
    nmmc_get_info(ctx, &info);
    const int nsl = info.nslices;

    mkdir(outdir, 0755);
    const std::string od = outdir;
    const long NS = opt.n_samp, NSL = NS * NL;
    // complete flags
    std::vector<int32_t> complete((size_t)nv1 * NL, 0);
    const bool have_flags = read_npy(join(od, "complete.npy"), "<i4", {nv1, NL}, complete.data(),
                                     complete.size() * sizeof(int32_t));
    // sample arrays (reloaded when resuming)
    const char* names[] = {"mags", "energies", "sub_mags", "sub4_mags", "mag_xs", "mag_ys", "mag_zs",
                           "sub_mag_xs", "sub_mag_ys", "sub_mag_zs", "sub4_mag_xs", "sub4_mag_ys", "sub4_mag_zs"};
    const int obs_of[] = {NMMC_OBS_ABSM, NMMC_OBS_E, NMMC_OBS_ABSSUBM, NMMC_OBS_ABSSUB4M, 1, 2, 3, 5, 6, 7, 9, 10, 11};
    const int narr = opt.is_ising ? 4 : 13;
    const size_t per = (size_t)nH * nT * NSL;
    std::vector<std::vector<float>> arr(narr, std::vector<float>(per, 0.0f));
    bool have_all = have_flags;
    for (int a = 0; a < narr; ++a)
        have_all &= read_npy(join(od, std::string(names[a]) + ".npy"), "<f4", {nH, nT, NSL}, arr[a].data(),
                             per * sizeof(float));
    const bool want_q = !opt.is_ising && !opt.distrib;   // output.cpp:235-246
    std::vector<float> tq(want_q ? (size_t)nH * nT * nsl * NSL : 0, 0.0f);
    if (want_q)
        have_all &= read_npy(join(od, "top_chars.npy"), "<f4", {nH, nT, nsl, NSL}, tq.data(), tq.size() * sizeof(float));
    // flags count only with every sample array of this run's shape present: otherwise start over
    if (!have_all) std::fill(complete.begin(), complete.end(), 0);

    // base chains: 20*EQ at Tmax (or a kept learned warm start, see GENERATOR), then EQ per v1
    // value and a fork into the inner chains
    std::vector<int> base(NL);
    for (int k = 0; k < NL; ++k) base[k] = k;
    {
        int initial = 20 * opt.eq_sweeps;
        std::string genfile;
        int ws_steps = 32, ws_sched = 0;
        if (!extra_keys(input_path, &genfile, &ws_steps, &ws_sched)) {
            rc = NMMC_ERR_INPUT;
            goto done;
        }
        if (!genfile.empty()) {
            int kept = 0;
            if ((rc = warm_start_base(ctx, join(wd, genfile), info.edge, base, Tmax, opt, ws_steps, ws_sched, seed,
                                      &kept)))
                goto done;
            if (kept) initial = 0;
            mkdir(outdir, 0755);
            const int32_t rec[2] = {kept, ws_steps};
            if (!write_npy(join(outdir, "warm_start.npy"), "<i4", {2}, rec, 4)) {
                rc = NMMC_ERR_IO;
                goto done;
            }
        }
        if ((rc = nmmc_sweep(ctx, base.data(), NL, initial))) goto done;
    }
    for (int i = b1; i != e1; i += s1) {
        for (int k = 0; k < NL; ++k)
            if ((rc = nmmc_change_v1(ctx, k, opt.protocol, v1[i]))) goto done;
        if ((rc = nmmc_sweep(ctx, base.data(), NL, opt.eq_sweeps))) goto done;
        for (int k = 0; k < NL; ++k)
            if ((rc = nmmc_fork(ctx, k, NL + i * NL + k))) goto done;
        if (verbose) printf("\rbase chains at v1[%d] = %g", i, v1[i]), fflush(stdout);
    }
    {
        std::vector<int> inner;
        for (int i = 0; i < nv1; ++i)
            for (int k = 0; k < NL; ++k)
                if (!complete[(size_t)i * NL + k]) inner.push_back(NL + i * NL + k);
        const int n = (int)inner.size();
        std::vector<double> obs((size_t)NS * n * NMMC_OBS_N), q(want_q ? (size_t)NS * n * nsl : 0);
        // /Av_Latt and /Sing_Latt of lattice 0 (main.cpp:174-177,236-254; output.cpp:100-150)
        std::vector<int> lat0;
        for (int c : inner)
            if ((c - NL) % NL == 0) lat0.push_back(c);
        const bool want_latt = !opt.distrib && !lat0.empty();
        const int nc = opt.is_ising ? 1 : 3;
        std::vector<long> lshape(info.dim, (long)info.edge);
        lshape.push_back(nc);
        std::vector<double> box((size_t)info.box_sites * 3);
        std::vector<float> latt((size_t)info.box_sites * nc);
        if (want_latt) {
            mkdir(join(od, "Av_Latt").c_str(), 0755);
            mkdir(join(od, "Sing_Latt").c_str(), 0755);
        }
        for (int j = b2; n > 0 && j != e2; j += s2) {
            for (int c : inner)
                if ((rc = nmmc_change_v2(ctx, c, opt.protocol, v2[j]))) goto done;
            if ((rc = nmmc_sweep(ctx, inner.data(), n, opt.eq_sweeps))) goto done;
            if (want_latt && (rc = nmmc_set_av_chains(ctx, lat0.data(), (int)lat0.size()))) goto done;
            if ((rc = nmmc_sample(ctx, inner.data(), n, opt.samp_sweeps, (int)NS, obs.data(), want_q ? q.data() : nullptr)))
                goto done;
            for (size_t l = 0; want_latt && l < lat0.size(); ++l) {
                const int i = (lat0[l] - NL) / NL;
                const int Hi = v1T ? j : i, Ti = v1T ? i : j;   // av_latt_name: protocol 4 as 2
                const std::string name = "T_" + std::to_string(Ti) + "-H_" + std::to_string(Hi) + ".npy";
                for (int which = 0; which < 2; ++which) {
                    rc = which ? nmmc_get_spins(ctx, lat0[l], box.data(), box.size() / 3)
                               : nmmc_get_av(ctx, lat0[l], box.data(), box.size() / 3);
                    if (rc) goto done;
                    // field_type::print (field_type.cpp:214-249): x slowest, then y (and z)
                    const long E = info.edge, ez = info.dim == 3 ? E : 1;
                    for (long x = 0; x < E; ++x)
                        for (long y = 0; y < E; ++y)
                            for (long z = 0; z < ez; ++z)
                                for (int k = 0; k < nc; ++k)
                                    latt[((x * E + y) * ez + z) * nc + k] = (float)box[(x + E * (y + E * z)) * 3 + k];
                    if (!write_npy(join(od, join(which ? "Sing_Latt" : "Av_Latt", name)), "<f4", lshape, latt.data(), 4)) {
                        rc = NMMC_ERR_IO;
                        goto done;
                    }
                }
            }
            for (int t = 0; t < n; ++t) {
                int i = (inner[t] - NL) / NL, k = (inner[t] - NL) % NL;
                int Hi = v1T ? j : i, Ti = v1T ? i : j;   // print_TD_h5: (H, T) from (var1, var2)
                for (long s = 0; s < NS; ++s) {
                    const double* o = &obs[((size_t)s * n + t) * NMMC_OBS_N];
                    size_t at = ((size_t)Hi * nT + Ti) * NSL + (size_t)k * NS + s;
                    for (int a = 0; a < narr; ++a) arr[a][at] = (float)o[obs_of[a]];
                    if (opt.is_ising) arr[0][at] = (float)fabs(o[1]);
                    if (want_q)
                        for (int z = 0; z < nsl; ++z)
                            tq[(((size_t)Hi * nT + Ti) * nsl + z) * NSL + (size_t)k * NS + s] =
                                (float)q[((size_t)s * n + t) * nsl + z];
                }
            }
            if (verbose) printf("\rsampled v2[%d] = %g for %d chains          ", j, v2[j], n), fflush(stdout);
            std::vector<long> shp = {nH, nT, NSL};
            for (int a = 0; a < narr; ++a)
                if (!write_npy(join(od, std::string(names[a]) + ".npy"), "<f4", shp, arr[a].data(), 4)) {
                    rc = NMMC_ERR_IO;
                    goto done;
                }
            if (want_q && !write_npy(join(od, "top_chars.npy"), "<f4", {nH, nT, nsl, NSL}, tq.data(), 4)) {
                rc = NMMC_ERR_IO;
                goto done;
            }
        }
        if (want_latt && (rc = nmmc_set_av_chains(ctx, nullptr, 0))) goto done;
        for (int c : inner) complete[(size_t)((c - NL) / NL) * NL + (c - NL) % NL] = 1;
        std::vector<float> tsf(Ts.begin(), Ts.end()), hsf(Hs.begin(), Hs.end());
        if (!write_npy(join(od, "Ts.npy"), "<f4", {nT}, tsf.data(), 4) ||
            !write_npy(join(od, "Hs.npy"), "<f4", {nH}, hsf.data(), 4) ||
            !write_npy(join(od, "complete.npy"), "<i4", {nv1, NL}, complete.data(), 4))
            rc = NMMC_ERR_IO;
    }
    if (verbose) printf("\n");
done:
    nmmc_destroy(ctx);
    return rc;
}
