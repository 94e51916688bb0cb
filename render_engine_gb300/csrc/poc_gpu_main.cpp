// Command-line front end with the reference's interface (cuda/poc_gpu.cu:1-9, 1286-1572):
//
//   poc_gpu_l3 timing  <scene.bin>
//   poc_gpu_l3 res     <scene.bin>
//   poc_gpu_l3 scen    <scene.bin> <nseeds>
//   poc_gpu_l3 scenf   <scene.bin> <nseeds> <scenarios.txt> [baseline budget]
//   poc_gpu_l3 quality <scene.bin> <nseeds> <budget1,budget2,...>
//   poc_gpu_l3 recon   <scene.bin> <nseeds>
//   poc_gpu_l3 taa     <scene.bin> <nseeds> <scenarios.txt>
//   poc_gpu_l3 prep    <mesh.msh> <scene.bin> [points]
//
// Same JSONL lines on stdout, same environment variables (BENCH_RAYONS, BENCH_DEBUG), so
// cuda/run_cuda.sh and cuda/analyse_cuda.py of the reference consume the output unchanged.
// The binary name fixes the scene light count like -DNLIGHTS does (poc_gpu.cu:755).  It is
// a client of the C ABI in include/rc_api.h and holds no CUDA code itself.
#include <sys/resource.h>
#include <time.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "rc_api.h"

#ifndef RC_CLI_NLIGHTS
#define RC_CLI_NLIGHTS 3
#endif

namespace {

struct Meth {
    std::string name;
    rc_method m;
};

rc_method mk(int mode, float nmax, float budget, bool deps = false, bool verify = false, bool oracle = false, int track_every = 1) {
    rc_method m;
    memset(&m, 0, sizeof m);
    m.mode = mode; m.nmax = nmax; m.budget = budget; m.deps = deps; m.verify = verify; m.oracle = oracle;
    m.track_every = track_every; m.nmax_resp = 8.f; m.ddgi_h = 0.97f; m.ddgi_thr = 0.25f; m.ddgi_clamp = 1; m.rays = 1.f;
    return m;
}

float g_rays = 1.f;
int g_debug = 0;

void die(rc_ctx* ctx, rc_status s, const char* what) {
    fprintf(stderr, "%s: %s (%s)\n", what, rc_status_string(s), ctx ? rc_last_error(ctx) : "");
    exit(s == RC_ERR_CUDA ? 2 : 1);
}
#define CHK(ctx, x, what)                 \
    do {                                  \
        rc_status s_ = (x);               \
        if (s_ != RC_OK) die(ctx, s_, what); \
    } while (0)

double cpu_seconds() {
    struct rusage u;
    getrusage(RUSAGE_SELF, &u);
    return u.ru_utime.tv_sec + u.ru_utime.tv_usec * 1e-6 + u.ru_stime.tv_sec + u.ru_stime.tv_usec * 1e-6;
}
double ram_mb() {
    struct rusage u;
    getrusage(RUSAGE_SELF, &u);
    return u.ru_maxrss / 1024.0;
}
double now_ms() {
    timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return t.tv_sec * 1000.0 + t.tv_nsec / 1e6;
}

std::vector<float> run(rc_ctx* ctx, const rc_method& m0, const std::vector<int>& seq, uint32_t seed, bool want_err, rc_timers* tm) {
    rc_method m = m0;
    m.rays = g_rays;
    std::vector<float> errs(seq.size());
    CHK(ctx, rc_run(ctx, &m, seq.data(), (int)seq.size(), seed, want_err ? 1 : 0, want_err ? errs.data() : nullptr, tm), "run");
    if (g_debug) {
        unsigned fl = 0;
        rc_device_flags(ctx, &fl);
        if (fl) fprintf(stderr, "[trace] device guard flags 0x%x\n", fl);
    }
    return errs;
}

std::vector<Meth> methods_quality(const std::vector<float>& budgets) {
    std::vector<Meth> M;
    char nm[160];
    for (float b : budgets) {
        for (int N : {8, 16, 32}) {
            snprintf(nm, sizeof nm, "Accumulation N=%d, %.2fx rayons", N, b);
            M.push_back({nm, mk(0, float(N), b)});
            snprintf(nm, sizeof nm, "Accumulation+parlampe N=%d, %.2fx rayons", N, b);
            rc_method r = mk(0, float(N), b); r.rescale = 1; M.push_back({nm, r});
        }
        for (int N : {16, 32, 64})
            for (int R : {4, 8}) {
                snprintf(nm, sizeof nm, "SHaRC N=%d resp=%d, %.2fx rayons", N, R, b);
                rc_method r = mk(0, float(N), b); r.resp_mask = 1; r.nmax_resp = float(R); r.rescale = 1; M.push_back({nm, r});
            }
        for (float h : {0.9f, 0.97f})
            for (float t : {0.25f, 0.5f, 1.0f})
                for (int cl : {0, 1})
                    for (int pl : {0, 1}) {
                        snprintf(nm, sizeof nm, "DDGI%s h=%.2f seuil=%.2f borne=%d, %.2fx rayons", pl ? "+parlampe" : "", h, t, cl, b);
                        rc_method r = mk(0, 64.f, b); r.ddgi = 1; r.ddgi_h = h; r.ddgi_thr = t; r.ddgi_clamp = cl; r.rescale = pl;
                        M.push_back({nm, r});
                    }
    }
    M.push_back({"Cache a dependances v3", mk(1, 64.f, 1.f, true, true, false, 1)});
    M.push_back({"Cache a dependances v3, suivi 1/4", mk(1, 64.f, 1.f, true, true, false, 4)});
    M.push_back({"Oracle", mk(1, 64.f, 1.f, false, false, true)});
    return M;
}

rc_method v4(bool memory, bool wake_verify, bool ramp) {
    rc_method r = mk(1, 64.f, 1.f, true, true, false, 4);
    r.memory = memory; r.wake_verify = wake_verify; r.ramp = ramp;
    return r;
}

void print_scen(const char* scen, const std::string& name, double pre, double post, int last, const std::vector<double>& curve) {
    printf("{\"type\":\"scen\",\"scen\":\"%s\",\"name\":\"%s\",\"pre\":%.5f,\"post\":%.5f,\"last\":%d,\"curve\":[", scen, name.c_str(), pre,
           post, last);
    for (size_t f = 0; f < curve.size(); ++f) printf("%s%.5f", f ? "," : "", curve[f]);
    printf("]}\n");
    fflush(stdout);
}

void run_scenarios(rc_ctx* ctx, const std::vector<std::pair<std::string, std::vector<std::pair<int, int>>>>& SC,
                   const std::vector<Meth>& M, int nseeds, uint32_t seed0) {
    for (auto& sc : SC) {
        std::vector<int> seq;
        for (auto& pr : sc.second)
            for (int k = 0; k < pr.second; ++k) seq.push_back(pr.first);
        if (seq.empty()) continue;
        int last = (int)seq.size() - sc.second.back().second;
        for (auto& m : M) {
            double pre = 0, post = 0;
            std::vector<double> curve(seq.size(), 0.0);
            for (int sd = 0; sd < nseeds; ++sd) {
                auto er = run(ctx, m.m, seq, seed0 + sd, true, nullptr);
                for (int f = last - 20; f < last; ++f) if (f >= 0 && f < (int)er.size()) pre += er[f] / 20.0 / nseeds;
                for (int f = last; f < last + 30; ++f) if (f >= 0 && f < (int)er.size()) post += er[f] / 30.0 / nseeds;
                for (size_t f = 0; f < seq.size(); ++f) curve[f] += er[f] / nseeds;
            }
            print_scen(sc.first.c_str(), m.name, pre, post, last, curve);
        }
    }
}

// One run with the per-point estimate of frames f0 .. f0 + nf - 1 added into sum / sq (the
// reference's k_accum_est after each such frame, poc_gpu.cu:698-703, 1003-1004): float
// sums, e * e fused into the square sum as the reference's compiled kernel does.
std::vector<float> run_recorded(rc_ctx* ctx, const rc_method& m0, const std::vector<int>& seq, uint32_t seed, int f0, int nf,
                                size_t np, int nl, std::vector<float>& sum, std::vector<float>& sq, std::vector<float>& lc) {
    rc_method m = m0;
    m.rays = g_rays;
    CHK(ctx, rc_run_begin(ctx, &m, seq[0], seed), "run");
    for (int f = 0; f < (int)seq.size(); ++f) {
        CHK(ctx, rc_frame(ctx, seq[f], 1), "frame");
        if (f < f0 || f >= f0 + nf) continue;
        CHK(ctx, rc_array_copy(ctx, RC_A_LC, lc.data(), lc.size() * sizeof(float), 0), "cache");
        int dormant = 0;
        CHK(ctx, rc_scalar_get(ctx, RC_S_DORMANT, &dormant), "dormant");
        float* s = sum.data() + (size_t)(f - f0) * np;
        float* q = sq.data() + (size_t)(f - f0) * np;
        for (size_t i = 0; i < np; ++i) {
            float e = 0.f;   // est_of (poc_gpu.cu:427-431)
            for (int l = 0; l < nl; ++l)
                if (!((dormant >> l) & 1)) e += lc[(size_t)nl * i + l];
            s[i] += e;
            q[i] = std::fmaf(e, e, q[i]);
        }
    }
    std::vector<float> errs(seq.size());
    int n = 0;
    CHK(ctx, rc_errors(ctx, errs.data(), (int)errs.size(), &n), "errors");
    errs.resize((size_t)n);
    return errs;
}

// Scenario file `name;state:frames,state:frames,...` (poc_gpu.cu:1376-1392, 1178-1187).
using Scenarios = std::vector<std::pair<std::string, std::vector<std::pair<int, int>>>>;
bool read_scenarios(const char* path, int NS, Scenarios& SC) {
    FILE* sf = fopen(path, "r");
    if (!sf) { fprintf(stderr, "fichier de scenarios %s\n", path); return false; }
    char line[512];
    while (fgets(line, sizeof line, sf)) {
        std::string L(line);
        while (!L.empty() && (L.back() == '\n' || L.back() == '\r')) L.pop_back();
        if (L.empty() || L[0] == '#') continue;
        size_t sc = L.find(';');
        if (sc == std::string::npos) continue;
        std::pair<std::string, std::vector<std::pair<int, int>>> x;
        x.first = L.substr(0, sc);
        std::string rest = L.substr(sc + 1);
        size_t pos = 0;
        while (pos < rest.size()) {
            size_t comma = rest.find(',', pos);
            if (comma == std::string::npos) comma = rest.size();
            std::string tok = rest.substr(pos, comma - pos);
            size_t colon = tok.find(':');
            int st = atoi(tok.substr(0, colon).c_str());
            int nf = colon == std::string::npos ? 0 : atoi(tok.substr(colon + 1).c_str());
            if (st < 0 || st >= NS) {
                fprintf(stderr, "scenario %s : etat %d hors limites\n", x.first.c_str(), st);
                fclose(sf);
                return false;
            }
            x.second.push_back({st, nf});
            pos = comma + 1;
        }
        SC.push_back(x);
    }
    fclose(sf);
    return true;
}

// taa mode (run_taa_mode, poc_gpu.cu:1175-1282): 8 accumulator variants per scenario, one
// JSONL line each with the 20-frame pre-event and 30-frame post-event errors and the curve.
int taa_mode(rc_ctx* ctx, int NS, const char* scen_file, int nseeds) {
    Scenarios SC;
    if (!read_scenarios(scen_file, NS, SC)) return 1;
    struct TM { std::string name; rc_taa_method m; };
    std::vector<TM> M;
    char nm[96];
    for (float a : {0.05f, 0.1f, 0.2f}) {
        snprintf(nm, sizeof nm, "TAA borne alpha=%.2f", a);
        M.push_back({nm, {a, 1.f, 0}});
    }
    M.push_back({"TAA simple alpha=0.10 (sans bornage)", {0.1f, 0.f, 0}});
    M.push_back({"TAA + detection aveugle", {0.1f, 1.f, 1}});
    M.push_back({"TAA + masque dependances", {0.1f, 1.f, 2}});
    M.push_back({"TAA + masque dependances verifie", {0.1f, 1.f, 3}});
    M.push_back({"TAA + masque oracle", {0.1f, 1.f, 4}});
    for (auto& sc : SC) {
        std::vector<int> seq;
        for (auto& pr : sc.second) for (int k = 0; k < pr.second; ++k) seq.push_back(pr.first);
        if (seq.empty()) continue;
        const int last = (int)seq.size() - sc.second.back().second;
        for (auto& m : M) {
            double pre = 0, post = 0;
            std::vector<double> curve(seq.size(), 0.0);
            for (int sd = 0; sd < nseeds; ++sd) {
                CHK(ctx, rc_taa_begin(ctx, &m.m, seq[0], 5000u + (uint32_t)sd), "taa");
                for (size_t f = 0; f < seq.size(); ++f) {
                    float e = 0.f;
                    CHK(ctx, rc_taa_frame(ctx, seq[f], &e), "taa frame");
                    curve[f] += (double)e / nseeds;
                    if ((int)f >= last - 20 && (int)f < last) pre += e / 20.0 / nseeds;
                    if ((int)f >= last && (int)f < last + 30) post += e / 30.0 / nseeds;
                }
            }
            printf("{\"type\":\"taa\",\"scen\":\"%s\",\"name\":\"%s\",\"pre\":%.5f,\"post\":%.5f,\"last\":%d,\"curve\":[", sc.first.c_str(),
                   m.name.c_str(), pre, post, last);
            for (size_t f = 0; f < curve.size(); ++f) printf("%s%.5f", f ? "," : "", curve[f]);
            printf("]}\n");
            fflush(stdout);
        }
    }
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 3) { fprintf(stderr, "usage\n"); return 1; }
    std::string mode = argv[1];
    if (const char* d = getenv("BENCH_DEBUG")) g_debug = atoi(d);
    if (const char* r = getenv("BENCH_RAYONS")) g_rays = std::max(0.25f, (float)atof(r));
    if (mode == "prep") {   // poc_gpu.cu:1304-1306, prep_mesh.cuh:303-531
        // poc_gpu_l3 places the reference's three lamps; poc_gpu_l8 places eight
        if (argc < 4) { fprintf(stderr, "usage : prep <maillage.mesh> <scene.bin> [points]\n"); return 1; }
        rc_config pc;
        memset(&pc, 0, sizeof pc);
        pc.expect_lights = RC_CLI_NLIGHTS;
        rc_ctx* pctx = nullptr;
        rc_status ps = rc_create(&pc, &pctx);
        if (ps != RC_OK) { fprintf(stderr, "CUDA: %s\n", rc_status_string(ps)); return 2; }
        rc_prep_report r;
        rc_prep_params pp;
        pp.target_points = argc > 4 ? atoi(argv[4]) : 300000;
        pp.lamps = RC_CLI_NLIGHTS;
        pp.seed = 1u;
        pp.ref_iterations = 0;
        ps = rc_prep_mesh_params(pctx, argv[2], argv[3], &pp, &r);
        if (ps != RC_OK) {
            fprintf(stderr, "prep: %s\n", rc_last_error(pctx));
            rc_destroy(pctx);
            return ps == RC_ERR_CUDA ? 2 : 1;
        }
        printf("{\"type\":\"prep\",\"triangles\":%d,\"np\":%d,\"cellule_m\":%.4f,\"zones\":%d,\"diag_m\":%.2f,\"cube_m\":%.2f,"
               "\"bvh_noeuds\":%d,\"points_valides\":%.4f,\"bruit_ref\":[",
               r.triangles, r.np, r.cell_m, r.zones, r.diag_m, r.cube_m, r.bvh_nodes, r.valid_fraction);
        for (int k = 0; k < r.ns; ++k) printf("%s%.5f", k ? "," : "", r.noise[k]);
        printf("],\"iterations_ref\":[");
        for (int k = 0; k < r.ns; ++k) printf("%s%d", k ? "," : "", r.iterations[k]);
        printf("],\"lampes\":[");
        for (int l = 0; l < r.nl; ++l) printf("%s[%.3f,%.3f,%.3f]", l ? "," : "", r.lights[l][0], r.lights[l][1], r.lights[l][2]);
        printf("],\"secondes\":%.1f}\n", r.seconds);
        rc_destroy(pctx);
        return 0;
    }
    rc_config cfg;
    memset(&cfg, 0, sizeof cfg);
    cfg.expect_lights = RC_CLI_NLIGHTS;
    rc_ctx* ctx = nullptr;
    rc_status s = rc_create(&cfg, &ctx);
    if (s != RC_OK) die(nullptr, s, "no usable GPU");
    rc_device_info dev0;
    CHK(ctx, rc_device_info_get(ctx, &dev0), "device");
    double r0 = ram_mb();
    CHK(ctx, rc_scene_load(ctx, argv[2]), "scene");
    // every state built before any mode runs, as the reference's load() does (the timing mode
    // must not share the GPU with a state build, and res reports the whole scene's memory)
    CHK(ctx, rc_scene_build_states(ctx), "state builds");
    CHK(ctx, rc_sync(ctx), "sync");
    rc_scene_info si;
    CHK(ctx, rc_scene_info_get(ctx, &si), "scene info");
    const int NS = si.ns, NL = si.nl;
    if (g_rays == 1.f)
        printf("{\"type\":\"scene\",\"np\":%d,\"nt\":%d,\"gpu\":\"%s\",\"mask_bits\":%d}\n", si.np, si.nt, dev0.name, 32 * si.nw);
    else
        printf("{\"type\":\"scene\",\"np\":%d,\"nt\":%d,\"gpu\":\"%s\",\"mask_bits\":%d,\"rayons_par_point\":%.2f,\"triangles_statiques\":%d}\n",
               si.np, si.nt, dev0.name, 32 * si.nw, g_rays, si.nst);
    fflush(stdout);
    if (mode == "res") {
        // poc_gpu.cu:1321-1343
        printf("{\"type\":\"vram\",\"contexte_mb\":%.1f,\"scene_mb\":%.1f,\"cache_tous_buffers_mb\":%.1f,\"ram_pic_mb\":%.1f,\"ram_debut_mb\":%.1f}\n",
               dev0.mem_used_mb, si.scene_bytes / 1048576.0, si.cache_bytes / 1048576.0, ram_mb(), r0);
        std::vector<int> seq;
        for (int st = 0; st < NS; ++st) for (int f = 0; f < 60; ++f) seq.push_back(st);
        std::vector<Meth> M;
        M.push_back({"Classique", mk(0, 16.f, 1.f)});
        { rc_method r = mk(0, 64.f, 1.f); r.resp_mask = 1; r.rescale = 1; M.push_back({"SHaRC responsive", r}); }
        M.push_back({"v3", mk(1, 64.f, 1.f, true, true, false, 4)});
        M.push_back({"v4-A2C", v4(true, true, true)});
        for (auto& m : M) {
            run(ctx, m.m, seq, 5, false, nullptr);
            double c0 = cpu_seconds(), t0 = now_ms();
            const int reps = 3;
            for (int k = 0; k < reps; ++k) run(ctx, m.m, seq, 9 + k, false, nullptr);
            CHK(ctx, rc_sync(ctx), "sync");
            double c1 = cpu_seconds(), t1 = now_ms();
            int frames = reps * (int)seq.size();
            printf("{\"type\":\"cpu\",\"name\":\"%s\",\"cpu_ms_par_frame\":%.4f,\"mur_ms_par_frame\":%.4f}\n", m.name.c_str(),
                   (c1 - c0) * 1000.0 / frames, (t1 - t0) / frames);
            fflush(stdout);
        }
    } else if (mode == "timing") {
        // poc_gpu.cu:1344-1367
        std::vector<int> seq;
        for (int st = 0; st < NS; ++st) for (int f = 0; f < 60; ++f) seq.push_back(st);
        std::vector<Meth> M;
        M.push_back({"Classique 1.0x", mk(0, 16.f, 1.f)});
        M.push_back({"Classique 2.0x", mk(0, 16.f, 2.f)});
        { rc_method r = mk(0, 32.f, 1.f); r.resp_mask = 1; r.rescale = 1; M.push_back({"SHaRC responsive 1.0x", r}); }
        { rc_method r = mk(0, 64.f, 1.f); r.ddgi = 1; r.rescale = 1; M.push_back({"DDGI 1.0x", r}); }
        M.push_back({"v3 sans suivi", mk(1, 64.f, 1.f, false, true, false)});
        M.push_back({"v3 complet", mk(1, 64.f, 1.f, true, true, false, 1)});
        M.push_back({"v3 suivi 1 frame sur 2", mk(1, 64.f, 1.f, true, true, false, 2)});
        M.push_back({"v3 suivi 1 frame sur 4", mk(1, 64.f, 1.f, true, true, false, 4)});
        M.push_back({"v4-A2C suivi 1/4", v4(true, true, true)});
        for (auto& m : M) {
            rc_timers warm;
            memset(&warm, 0, sizeof warm);
            run(ctx, m.m, seq, 7, false, &warm);
            rc_timers t;
            memset(&t, 0, sizeof t);
            for (int rep = 0; rep < 3; ++rep) run(ctx, m.m, seq, 11 + rep, false, &t);
            printf("{\"type\":\"timing\",\"name\":\"%s\",\"trace\":%.5f,\"decide\":%.5f,\"update\":%.5f,\"swap\":%.5f,\"event\":%.5f}\n",
                   m.name.c_str(), t.trace / t.frames, t.decide / t.frames, t.update / t.frames, t.swap / t.frames,
                   t.events ? t.event / t.events : 0.0);
            fflush(stdout);
        }
    } else if (mode == "taa") {
        // poc_gpu.cu:1368-1370
        if (argc < 5) { fprintf(stderr, "usage : taa <scene.bin> <nseeds> <scenarios.txt>\n"); return 1; }
        if (si.fmt == 3) { fprintf(stderr, "mode taa non supporte sur les scenes maillees\n"); return 1; }
        return taa_mode(ctx, NS, argv[4], atoi(argv[3]));
    } else if (mode == "scenf") {
        // poc_gpu.cu:1371-1437
        if (argc < 5) { fprintf(stderr, "usage : scenf <scene.bin> <nseeds> <scenarios.txt> [budget]\n"); return 1; }
        int nseeds = atoi(argv[3]);
        Scenarios SC;
        if (!read_scenarios(argv[4], NS, SC)) return 1;
        // lights whose intensity differs from state 0 are "responsive" for SHaRC (poc_gpu.cu:1396-1397)
        std::vector<float> in0(NL), ink(NL);
        int dyn = 0;
        CHK(ctx, rc_state_lights(ctx, 0, in0.data(), NL), "lights");
        for (int st = 1; st < NS; ++st) {
            CHK(ctx, rc_state_lights(ctx, st, ink.data(), NL), "lights");
            for (int l = 0; l < NL; ++l) if (ink[l] != in0[l]) dyn |= 1 << l;
        }
        float bS = 1.57f, bA = 1.53f;
        if (argc > 5) bS = bA = (float)atof(argv[5]);
        char nm[160];
        auto nmf = [&](const char* fmt, float b) { snprintf(nm, sizeof nm, fmt, b); return std::string(nm); };
        std::vector<Meth> M;
        auto sharc = [&](float b) { rc_method r = mk(0, 64.f, b); r.resp_mask = dyn; r.nmax_resp = 8.f; r.rescale = 1; return r; };
        auto accum = [&](float N, float b) { rc_method r = mk(0, N, b); r.rescale = 1; return r; };
        M.push_back({nmf("SHaRC N=64 resp=8, %.2fx", bS), sharc(bS)});
        { rc_method r = sharc(bS); r.memory = 1; M.push_back({nmf("SHaRC + memoire naive, %.2fx", bS), r}); }
        M.push_back({nmf("Accumulation+parlampe N=32, %.2fx", bA), accum(32.f, bA)});
        { rc_method r = accum(32.f, bA); r.memory = 1; M.push_back({nmf("Accum+parlampe + memoire naive N=32, %.2fx", bA), r}); }
        { rc_method r = accum(64.f, bA); r.memory = 1; M.push_back({nmf("Accum+parlampe + memoire naive N=64, %.2fx", bA), r}); }
        { rc_method r = sharc(bS); r.memory = 1; r.snaps = 1; M.push_back({nmf("SHaRC + memoire + instantanes, %.2fx", bS), r}); }
        { rc_method r = accum(32.f, bA); r.memory = 1; r.snaps = 1; M.push_back({nmf("Accum + memoire + instantanes N=32, %.2fx", bA), r}); }
        { rc_method r = accum(64.f, bA); r.memory = 1; r.snaps = 1; M.push_back({nmf("Accum + memoire + instantanes N=64, %.2fx", bA), r}); }
        M.push_back({"Oracle", mk(1, 64.f, 1.f, false, false, true)});
        M.push_back({"v3", mk(1, 64.f, 1.f, true, true, false, 4)});
        M.push_back({"v4-A2C memoire verifiee+rampe", v4(true, true, true)});
        { rc_method r = v4(true, true, true); r.snaps = 1; r.snap_verify = 1; M.push_back({"v5-A instantanes verifies", r}); }
        { rc_method r = v4(true, true, true); r.snaps = 1; M.push_back({"v5-A instantanes", r}); }
        { rc_method r = v4(true, true, true); r.snaps = 1; r.proj = 1; M.push_back({"v5-AB instantanes+projection", r}); }
        run_scenarios(ctx, SC, M, nseeds, 3000);
    } else if (mode == "scen") {
        // poc_gpu.cu:1438-1488
        int nseeds = argc > 3 ? atoi(argv[3]) : 1;
        std::vector<std::pair<std::string, std::vector<std::pair<int, int>>>> SC = {
            {"R1 allumee-eteinte-rallumee", {{0, 50}, {1, 30}, {0, 50}}},
            {"R2 allumee-eteinte-porte-rallumee", {{0, 40}, {1, 20}, {2, 20}, {3, 50}}},
            {"R3 porte ouverte-fermee-rouverte", {{0, 50}, {3, 30}, {0, 50}}},
            {"I1 lampe eteinte", {{0, 50}, {1, 50}}},
            {"I2 porte", {{1, 50}, {2, 50}}},
            {"I3 lampe allumee 1re fois", {{2, 50}, {3, 50}}},
            {"I4 boite", {{3, 50}, {4, 50}}},
        };
        for (auto& sc : SC)
            for (auto& pr : sc.second)
                if (pr.first >= NS) { fprintf(stderr, "mode scen : la scene a %d etats\n", NS); return 1; }
        std::vector<Meth> M;
        auto sharc = [](float b) { rc_method r = mk(0, 64.f, b); r.resp_mask = 1; r.nmax_resp = 8.f; r.rescale = 1; return r; };
        auto accum = [](float N, float b) { rc_method r = mk(0, N, b); r.rescale = 1; return r; };
        M.push_back({"SHaRC N=64 resp=8, 1.57x", sharc(1.57f)});
        M.push_back({"Accumulation+parlampe N=32, 1.53x", accum(32.f, 1.53f)});
        { rc_method r = sharc(1.57f); r.memory = 1; M.push_back({"SHaRC + memoire naive, 1.57x", r}); }
        { rc_method r = accum(32.f, 1.53f); r.memory = 1; M.push_back({"Accum+parlampe + memoire naive N=32, 1.53x", r}); }
        { rc_method r = accum(64.f, 1.53f); r.memory = 1; M.push_back({"Accum+parlampe + memoire naive N=64, 1.53x", r}); }
        { rc_method r = sharc(1.57f); r.memory = 1; r.snaps = 1; M.push_back({"SHaRC + memoire + instantanes, 1.57x", r}); }
        { rc_method r = accum(32.f, 1.53f); r.memory = 1; r.snaps = 1; M.push_back({"Accum + memoire + instantanes N=32, 1.53x", r}); }
        { rc_method r = accum(64.f, 1.53f); r.memory = 1; r.snaps = 1; M.push_back({"Accum + memoire + instantanes N=64, 1.53x", r}); }
        M.push_back({"Oracle", mk(1, 64.f, 1.f, false, false, true)});
        M.push_back({"v3", mk(1, 64.f, 1.f, true, true, false, 4)});
        M.push_back({"v4-A memoire", v4(true, false, false)});
        M.push_back({"v4-C rampe", v4(false, false, true)});
        M.push_back({"v4-AC memoire+rampe", v4(true, false, true)});
        M.push_back({"v4-A2 memoire verifiee", v4(true, true, false)});
        M.push_back({"v4-A2C memoire verifiee+rampe", v4(true, true, true)});
        { rc_method r = v4(true, true, true); r.snaps = 1; r.snap_verify = 1; M.push_back({"v5-A instantanes verifies", r}); }
        { rc_method r = v4(true, true, true); r.snaps = 1; M.push_back({"v5-A instantanes", r}); }
        { rc_method r = v4(true, true, true); r.snaps = 1; r.proj = 1; M.push_back({"v5-AB instantanes+projection", r}); }
        run_scenarios(ctx, SC, M, nseeds, 2000);
    } else if (mode == "quality") {
        // poc_gpu.cu:1549-1568
        if (argc < 5) { fprintf(stderr, "usage : quality <scene.bin> <nseeds> <budgets>\n"); return 1; }
        int nseeds = atoi(argv[3]);
        std::vector<float> budgets;
        for (char* tok = strtok(argv[4], ","); tok; tok = strtok(nullptr, ",")) budgets.push_back((float)atof(tok));
        for (auto& m : methods_quality(budgets)) {
            for (int e = 0; e < NS - 1; ++e) {
                std::vector<int> seq(100, e);
                for (int f = 50; f < 100; ++f) seq[f] = e + 1;
                double pre = 0, post = 0;
                for (int sd = 0; sd < nseeds; ++sd) {
                    auto er = run(ctx, m.m, seq, 1000 + sd, true, nullptr);
                    for (int f = 30; f < 50; ++f) pre += er[f] / 20.0 / nseeds;
                    for (int f = 50; f < 80; ++f) post += er[f] / 30.0 / nseeds;
                }
                printf("{\"type\":\"quality\",\"name\":\"%s\",\"budget\":%.3f,\"event\":%d,\"pre\":%.5f,\"post\":%.5f}\n", m.name.c_str(),
                       m.m.budget, e, pre, post);
            }
            fflush(stdout);
        }
    } else if (mode == "recon") {
        // poc_gpu.cu:1489-1547: per-seed curves, then bias^2 and variance of the estimate over
        // frames 45..99 in three categories of points (relative change of the reference > 20 %,
        // 5-20 %, < 5 %)
        if (argc < 4) { fprintf(stderr, "usage : recon <scene.bin> <nseeds>\n"); return 1; }
        int nseeds = atoi(argv[3]);
        const int F0 = 45, NF = 55;
        std::vector<Meth> M;
        M.push_back({"Cache a dependances v3, suivi 1/4", mk(1, 64.f, 1.f, true, true, false, 4)});
        { rc_method r = mk(0, 64.f, 1.52f); r.resp_mask = 1; r.nmax_resp = 8.f; r.rescale = 1; M.push_back({"SHaRC N=64 resp=8, 1.52x", r}); }
        { rc_method r = mk(0, 32.f, 1.51f); r.rescale = 1; M.push_back({"Accumulation+parlampe N=32, 1.51x", r}); }
        M.push_back({"Oracle", mk(1, 64.f, 1.f, false, false, true)});
        const size_t Np = (size_t)si.np;
        std::vector<float> hsum((size_t)NF * Np), hsq((size_t)NF * Np), lc(Np * (size_t)NL);
        std::vector<float> rold(Np), rnew(Np);
        std::vector<uint8_t> val(Np);
        for (auto& m : M)
            for (int e = 0; e < NS - 1; ++e) {
                std::vector<int> seq(100, e);
                for (int f = 50; f < 100; ++f) seq[f] = e + 1;
                std::fill(hsum.begin(), hsum.end(), 0.f);
                std::fill(hsq.begin(), hsq.end(), 0.f);
                printf("{\"type\":\"recon_seeds\",\"name\":\"%s\",\"event\":%d,\"curves\":[", m.name.c_str(), e);
                for (int sd = 0; sd < nseeds; ++sd) {
                    auto er = run_recorded(ctx, m.m, seq, 1000 + sd, F0, NF, Np, NL, hsum, hsq, lc);
                    printf("%s[", sd ? "," : "");
                    for (size_t f = 0; f < er.size(); ++f) printf("%s%.5f", f ? "," : "", er[f]);
                    printf("]");
                }
                printf("]}\n");
                CHK(ctx, rc_state_array_copy(ctx, e, RC_SA_REF, rold.data(), Np * 4), "reference");
                CHK(ctx, rc_state_array_copy(ctx, e + 1, RC_SA_REF, rnew.data(), Np * 4), "reference");
                CHK(ctx, rc_state_array_copy(ctx, e + 1, RC_SA_VALID, val.data(), Np), "valid");
                double mref = 0;
                int nv = 0;
                std::vector<int> cat(Np, -1);
                for (size_t i = 0; i < Np; ++i)
                    if (val[i]) {
                        double rel = fabs(rnew[i] - rold[i]) / (rold[i] + 1e-2);
                        cat[i] = rel > 0.2 ? 0 : (rel > 0.05 ? 1 : 2);
                        mref += rnew[i];
                        nv++;
                    }
                mref /= nv;
                printf("{\"type\":\"recon_bv\",\"name\":\"%s\",\"event\":%d,\"f0\":%d,\"mref\":%.6f,\"cats\":[", m.name.c_str(), e, F0, mref);
                for (int k = 0; k < 3; ++k) {
                    int cnt = 0;
                    for (size_t i = 0; i < Np; ++i) cnt += cat[i] == k;
                    printf("%s{\"n\":%d,\"bias2\":[", k ? "," : "", cnt);
                    std::vector<double> var(NF);
                    for (int f = 0; f < NF; ++f) {
                        double b2 = 0, v = 0;
                        for (size_t i = 0; i < Np; ++i)
                            if (cat[i] == k) {
                                double mu = hsum[f * Np + i] / nseeds;
                                double vv = hsq[f * Np + i] / nseeds - mu * mu;
                                b2 += (mu - rnew[i]) * (mu - rnew[i]);
                                v += vv > 0 ? vv : 0;
                            }
                        printf("%s%.6e", f ? "," : "", cnt ? b2 / cnt : 0.0);
                        var[f] = cnt ? v / cnt : 0.0;
                    }
                    printf("],\"var\":[");
                    for (int f = 0; f < NF; ++f) printf("%s%.6e", f ? "," : "", var[f]);
                    printf("]}");
                }
                printf("]}\n");
                fflush(stdout);
            }
    } else {
        fprintf(stderr, "mode inconnu : %s\n", mode.c_str());
        rc_destroy(ctx);
        return 1;
    }
    rc_destroy(ctx);
    return 0;
}
