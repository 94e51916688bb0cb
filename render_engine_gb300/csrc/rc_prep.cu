// Scene preparation: the reference's `prep` mode (cuda/prep_mesh.cuh:303-531), mesh -> format-3
// scene with converged references.  Host steps restated in this file's own code (the same
// algorithm, so that a mesh gives the scene the reference prepares from it):
//   1. binned-SAH BVH over the static triangles (prep_mesh.cuh:42-114);
//   2. cache points: a SHaRC-style cell grid (cell h, dominant normal bucket) sampled on the
//      triangles, h adjusted towards the requested point count (:116-157, :331-375);
//   3. three lamps and a movable cube placed in free space found by probe rays (:377-436);
//   4. five states (lamps on / off, cube moved) and the transit voxels of every event
//      (:437-441, :242-297);
//   5. direct light normalised to a mean of 1 in state 0, then converged references by the
//      two-chain stochastic Jacobi (:463-518).
// The GPU does the probe rays (probe_free_space, the frames' BVH traversal), the per-state
// build and the references (rc_reference_build) through a context.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

#include "../../include/rc_api.h"
#include "rc_internal.h"

namespace rc {
// defined with the context (rc_runtime.cu)
rc_status ctx_fail(rc_ctx* ctx, rc_status s, const char* fmt, ...);
rc_status ctx_probe_free_space(rc_ctx* ctx, const std::vector<float>& ST, const std::vector<float>& STN, const float* BN, int nnodes,
                               const std::vector<float>& C, float diag, std::vector<float>& out);
}  // namespace rc

namespace {

struct Mesh {
    int nt = 0;
    std::vector<float> V;      // 9 per triangle
    std::vector<float> alb;
    std::vector<uint8_t> ds;   // double-sided
};

// MSH1: "MSH1", int32 triangle count, 9 floats per triangle, one albedo per triangle, one
// double-sided byte per triangle (prep_mesh.cuh:22-29)
bool read_msh1(const char* path, Mesh& M, std::string& err) {
    FILE* f = fopen(path, "rb");
    if (!f) { err = std::string("mesh ") + path + " cannot be read"; return false; }
    char magic[4];
    int nt = 0;
    bool ok = fread(magic, 1, 4, f) == 4 && memcmp(magic, "MSH1", 4) == 0 && fread(&nt, 4, 1, f) == 1 && nt > 0 && nt < (1 << 28);
    if (ok) {
        M.nt = nt;
        M.V.resize(9 * (size_t)nt);
        M.alb.resize(nt);
        M.ds.resize(nt);
        ok = fread(M.V.data(), 4, M.V.size(), f) == M.V.size() && fread(M.alb.data(), 4, M.alb.size(), f) == M.alb.size() &&
             fread(M.ds.data(), 1, M.ds.size(), f) == M.ds.size();
    }
    fclose(f);
    if (!ok) err = std::string("mesh ") + path + ": not an MSH1 file or truncated";
    return ok;
}

uint64_t mix64(uint64_t x) {   // poc_gpu.cu:260-262
    x ^= x >> 30; x *= 0xbf58476d1ce4e5b9ull; x ^= x >> 27; x *= 0x94d049bb133111ebull; x ^= x >> 31;
    return x;
}

// the preparation's host generator (prep_mesh.cuh:32-36): mix64 stream, 24-bit uniforms
struct Rng {
    uint64_t s;
    explicit Rng(uint64_t x) : s(mix64(x * 0x9E3779B97F4A7C15ull + 1)) {}
    float u() {
        s = mix64(s + 0x9E3779B97F4A7C15ull);
        return (float)(s >> 40) * (1.0f / 16777216.0f);
    }
};

int normal_bucket(float nx, float ny, float nz) {   // poc_gpu.cu:251-256
    const float ax = fabsf(nx), ay = fabsf(ny), az = fabsf(nz);
    if (ax >= ay && ax >= az) return nx > 0.f ? 0 : 1;
    if (ay >= az) return ny > 0.f ? 2 : 3;
    return nz > 0.f ? 4 : 5;
}
uint64_t cell_key(int cx, int cy, int cz, int b) {   // poc_gpu.cu:257-259
    uint64_t k = (uint64_t)(cx & 0xFFFFF);
    k = (k << 20) | (uint64_t)(cy & 0xFFFFF);
    k = (k << 20) | (uint64_t)(cz & 0xFFFFF);
    return ((k << 3) | (uint64_t)b) + 1ull;
}
void key_cell(uint64_t k, int& cx, int& cy, int& cz, int& b) {
    k -= 1ull;
    b = (int)(k & 7ull);
    cz = (int)((k >> 3) & 0xFFFFFull);
    cy = (int)((k >> 23) & 0xFFFFFull);
    cx = (int)((k >> 43) & 0xFFFFFull);
}
uint64_t morton_spread(uint64_t x) {   // 21 bits to every third bit
    x &= 0x1fffffull;
    x = (x | x << 32) & 0x1f00000000ffffull;
    x = (x | x << 16) & 0x1f0000ff0000ffull;
    x = (x | x << 8) & 0x100f00f00f00f00full;
    x = (x | x << 4) & 0x10c30c30c30c30c3ull;
    x = (x | x << 2) & 0x1249249249249249ull;
    return x;
}

struct Node { float lo[3]; int lf; float hi[3]; int cnt; };   // the two float4 the traversal reads
static_assert(sizeof(Node) == 32, "BVH node: 32 bytes");

float box_area(const float* lo, const float* hi) {
    const float d0 = hi[0] - lo[0], d1 = hi[1] - lo[1], d2 = hi[2] - lo[2];
    return d0 < 0 ? 0.f : 2.f * (d0 * d1 + d1 * d2 + d2 * d0);
}

// Binned SAH (16 bins on the widest centroid axis), leaves of at most 4 triangles (64 when the
// centroids coincide), depth at most 56, median split when SAH finds no split; the two
// children of an inner node are adjacent (left = lf, right = lf + 1).
void build_bvh(const Mesh& M, std::vector<Node>& nodes, std::vector<int>& order) {
    const int n = M.nt;
    order.resize(n);
    std::iota(order.begin(), order.end(), 0);
    std::vector<float> cen(3 * (size_t)n), tlo(3 * (size_t)n), thi(3 * (size_t)n);
    for (int t = 0; t < n; ++t)
        for (int a = 0; a < 3; ++a) {
            const float x0 = M.V[9 * (size_t)t + a], x1 = M.V[9 * (size_t)t + 3 + a], x2 = M.V[9 * (size_t)t + 6 + a];
            tlo[3 * (size_t)t + a] = std::min(x0, std::min(x1, x2));
            thi[3 * (size_t)t + a] = std::max(x0, std::max(x1, x2));
            cen[3 * (size_t)t + a] = 0.5f * (tlo[3 * (size_t)t + a] + thi[3 * (size_t)t + a]);
        }
    nodes.clear();
    nodes.reserve(2 * (size_t)n + 1);
    nodes.push_back(Node{});
    struct Item { int node, start, count, depth; };
    std::vector<Item> work{{0, 0, n, 0}};
    constexpr int NB = 16;
    while (!work.empty()) {
        const Item it = work.back();
        work.pop_back();
        float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
        float clo[3] = {1e30f, 1e30f, 1e30f}, chi[3] = {-1e30f, -1e30f, -1e30f};
        for (int k = it.start; k < it.start + it.count; ++k) {
            const int t = order[k];
            for (int a = 0; a < 3; ++a) {
                lo[a] = std::min(lo[a], tlo[3 * (size_t)t + a]);
                hi[a] = std::max(hi[a], thi[3 * (size_t)t + a]);
                clo[a] = std::min(clo[a], cen[3 * (size_t)t + a]);
                chi[a] = std::max(chi[a], cen[3 * (size_t)t + a]);
            }
        }
        for (int a = 0; a < 3; ++a) {
            nodes[it.node].lo[a] = lo[a];
            nodes[it.node].hi[a] = hi[a];
        }
        auto leaf = [&]() { nodes[it.node].lf = it.start; nodes[it.node].cnt = it.count; };
        int ax = 0;
        for (int a = 1; a < 3; ++a)
            if (chi[a] - clo[a] > chi[ax] - clo[ax]) ax = a;
        const float ext = chi[ax] - clo[ax];
        if ((it.count <= 4 || it.depth >= 56 || ext < 1e-7f) && (it.count <= 64 || it.depth >= 56)) { leaf(); continue; }
        int mid = -1;
        if (ext >= 1e-7f) {
            auto bin_of = [&](int t) { return std::min(NB - 1, (int)((cen[3 * (size_t)t + ax] - clo[ax]) / ext * NB)); };
            int bc[NB] = {0};
            float blo[NB][3], bhi[NB][3];
            for (int b = 0; b < NB; ++b)
                for (int a = 0; a < 3; ++a) { blo[b][a] = 1e30f; bhi[b][a] = -1e30f; }
            for (int k = it.start; k < it.start + it.count; ++k) {
                const int t = order[k], b = bin_of(t);
                bc[b]++;
                for (int a = 0; a < 3; ++a) {
                    blo[b][a] = std::min(blo[b][a], tlo[3 * (size_t)t + a]);
                    bhi[b][a] = std::max(bhi[b][a], thi[3 * (size_t)t + a]);
                }
            }
            float best = 1e30f;
            int split = -1;
            for (int sb = 1; sb < NB; ++sb) {
                float l0[3] = {1e30f, 1e30f, 1e30f}, l1[3] = {-1e30f, -1e30f, -1e30f};
                float r0[3] = {1e30f, 1e30f, 1e30f}, r1[3] = {-1e30f, -1e30f, -1e30f};
                int nl = 0, nr = 0;
                for (int b = 0; b < NB; ++b) {
                    float* x0 = b < sb ? l0 : r0;
                    float* x1 = b < sb ? l1 : r1;
                    (b < sb ? nl : nr) += bc[b];
                    for (int a = 0; a < 3; ++a) { x0[a] = std::min(x0[a], blo[b][a]); x1[a] = std::max(x1[a], bhi[b][a]); }
                }
                if (!nl || !nr) continue;
                const float cost = nl * box_area(l0, l1) + nr * box_area(r0, r1);
                if (cost < best) { best = cost; split = sb; }
            }
            const float leaf_cost = it.count * box_area(lo, hi);
            if (split > 0 && !(it.count <= 4 && best >= leaf_cost)) {
                auto pm = std::partition(order.begin() + it.start, order.begin() + it.start + it.count,
                                         [&](int t) { return bin_of(t) < split; });
                mid = (int)(pm - order.begin());
            } else if (it.count <= 4) {
                leaf();
                continue;
            }
        }
        if (mid <= it.start || mid >= it.start + it.count) {
            mid = it.start + it.count / 2;
            std::nth_element(order.begin() + it.start, order.begin() + mid, order.begin() + it.start + it.count,
                             [&](int a, int b) { return cen[3 * (size_t)a + ax] < cen[3 * (size_t)b + ax]; });
        }
        const int left = (int)nodes.size();
        nodes.push_back(Node{});
        nodes.push_back(Node{});
        nodes[it.node].lf = left;
        nodes[it.node].cnt = 0;
        work.push_back({left, it.start, mid - it.start, it.depth + 1});
        work.push_back({left + 1, mid, it.start + it.count - mid, it.depth + 1});
    }
}

struct Cell { float p[3]; float d2; float n[3]; double asum, wsum; };

// Points on every triangle (its centroid, then uniform samples: about 4 per h^2 of area, seeded
// by the triangle index), binned into cells of side h from lo with the normal's bucket (both
// sides for a double-sided triangle); a cell keeps its sample closest to the cell centre and
// the area-weighted mean albedo.
void sample_cells(const Mesh& M, float h, const float lo[3], std::unordered_map<uint64_t, Cell>& cells) {
    cells.clear();
    for (int t = 0; t < M.nt; ++t) {
        const float* v = &M.V[9 * (size_t)t];
        const float e1[3] = {v[3] - v[0], v[4] - v[1], v[5] - v[2]}, e2[3] = {v[6] - v[0], v[7] - v[1], v[8] - v[2]};
        const float cr[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        const float l = sqrtf(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
        if (l < 1e-12f) continue;
        const float ar = 0.5f * l, n[3] = {cr[0] / l, cr[1] / l, cr[2] / l};
        const int ns = (int)std::min(1e6, std::max(1.0, std::ceil(ar / (h * h) * 4.0)));
        Rng r((uint64_t)t);
        const int sides = M.ds[t] ? 2 : 1;
        for (int k = 0; k < ns; ++k) {
            float a = 1.f / 3.f, b = 1.f / 3.f;
            if (k > 0) {
                a = r.u();
                b = r.u();
                if (a + b > 1.f) { a = 1.f - a; b = 1.f - b; }
            }
            const float P[3] = {v[0] + e1[0] * a + e2[0] * b, v[1] + e1[1] * a + e2[1] * b, v[2] + e1[2] * a + e2[2] * b};
            int c[3];
            float d2 = 0.f;
            for (int x = 0; x < 3; ++x) {
                c[x] = (int)floorf((P[x] - lo[x]) / h);
                const float cc = lo[x] + (c[x] + 0.5f) * h;
                d2 += (P[x] - cc) * (P[x] - cc);
            }
            for (int sd = 0; sd < sides; ++sd) {
                const float nn[3] = {sd ? -n[0] : n[0], sd ? -n[1] : n[1], sd ? -n[2] : n[2]};
                const uint64_t key = cell_key(c[0], c[1], c[2], normal_bucket(nn[0], nn[1], nn[2]));
                auto ins = cells.try_emplace(key, Cell{{0, 0, 0}, 1e30f, {0, 0, 1}, 0.0, 0.0});
                Cell& cl = ins.first->second;
                if (d2 < cl.d2) {
                    cl.d2 = d2;
                    for (int x = 0; x < 3; ++x) { cl.p[x] = P[x]; cl.n[x] = nn[x]; }
                }
                cl.asum += (double)M.alb[t] * ar / ns;
                cl.wsum += (double)ar / ns;
            }
        }
    }
}

struct Prepared {
    float lo[3], ext[3], h = 0.f;
    std::vector<float> ST, STN;
    std::vector<Node> BN;
    std::vector<uint64_t> HK;
    std::vector<int> HV;
    int npst = 0, nbox = 0, NR = 0, bnu = 0;
    std::vector<float> L, A;
    std::vector<int> region;
    std::vector<float> Pst, Nst;
    std::vector<std::vector<float>> inten;
    std::vector<int> boxpos;
    float boxc[2][3], boxe = 0.f;
    std::vector<std::vector<float>> ref, Pw;
    std::vector<std::vector<uint8_t>> valid;
};

constexpr int NLP = 3;                  // the preparation places three lamps (prep_mesh.cuh:304)
constexpr int GVX = 8, GVY = 4, GVZ = 4;   // transit grid of the reference build for event voxels

int host_vox(const Prepared& m, const float* p) {   // poc_gpu.cu:713-718
    const int i = std::min(std::max(int((p[0] - m.lo[0]) / m.ext[0] * GVX), 0), GVX - 1);
    const int j = std::min(std::max(int((p[1] - m.lo[1]) / m.ext[1] * GVY), 0), GVY - 1);
    const int k = std::min(std::max(int((p[2] - m.lo[2]) / m.ext[2] * GVZ), 0), GVZ - 1);
    return (k * GVY + j) * GVX + i;
}

// the cube's six faces as (o, u, v, n) with u x v along the outward normal (prep_mesh.cuh:229-240)
void cube_quads(const float c[3], float e, float Q[72]) {
    const float E = 2.f * e;
    const float F[6][12] = {{c[0] + e, c[1] - e, c[2] - e, 0, E, 0, 0, 0, E, 1, 0, 0},
                            {c[0] - e, c[1] - e, c[2] - e, 0, 0, E, 0, E, 0, -1, 0, 0},
                            {c[0] - e, c[1] + e, c[2] - e, 0, 0, E, E, 0, 0, 0, 1, 0},
                            {c[0] - e, c[1] - e, c[2] - e, E, 0, 0, 0, 0, E, 0, -1, 0},
                            {c[0] - e, c[1] - e, c[2] + e, E, 0, 0, 0, E, 0, 0, 0, 1},
                            {c[0] - e, c[1] - e, c[2] - e, 0, E, 0, E, 0, 0, 0, 0, -1}};
    memcpy(Q, F, sizeof F);
}

// Format-3 scene bytes (the layout poc_gpu.cu:751-801 reads; writer prep_mesh.cuh:242-297)
std::vector<uint8_t> scene_bytes(const Prepared& m, bool with_ref) {
    std::vector<uint8_t> out;
    auto W = [&](const void* p, size_t n) { out.insert(out.end(), (const uint8_t*)p, (const uint8_t*)p + n); };
    const int NS = (int)m.inten.size(), Np = m.npst + m.nbox;
    const int hdr[8] = {Np, 6, 12, NS, NLP, m.NR, with_ref ? 1 : 0, 3};
    W(hdr, 32);
    W(m.lo, 12);
    W(m.ext, 12);
    W(&m.h, 4);
    const int mm[4] = {(int)(m.ST.size() / 9), (int)m.BN.size(), (int)m.HK.size(), m.npst};
    W(mm, 16);
    W(m.ST.data(), m.ST.size() * 4);
    W(m.STN.data(), m.STN.size() * 4);
    W(m.BN.data(), m.BN.size() * sizeof(Node));
    W(m.HK.data(), m.HK.size() * 8);
    W(m.HV.data(), m.HV.size() * 4);
    W(m.L.data(), m.L.size() * 4);
    W(m.A.data(), m.A.size() * 4);
    W(m.region.data(), m.region.size() * 4);
    for (int si = 0; si < NS; ++si) {
        std::vector<float> P(m.Pst), N(m.Nst);
        float Q[72];
        cube_quads(m.boxc[m.boxpos[si]], m.boxe, Q);
        std::vector<int> dims, off;
        for (int q = 0; q < 6; ++q) {
            dims.push_back(m.bnu);
            dims.push_back(m.bnu);
            off.push_back(m.npst + q * m.bnu * m.bnu);
            for (int iv = 0; iv < m.bnu; ++iv)
                for (int iu = 0; iu < m.bnu; ++iu)
                    for (int x = 0; x < 3; ++x) {
                        P.push_back(Q[12 * q + x] + Q[12 * q + 3 + x] * (iu + 0.5f) / m.bnu + Q[12 * q + 6 + x] * (iv + 0.5f) / m.bnu);
                        N.push_back(Q[12 * q + 9 + x]);
                    }
        }
        std::vector<float> T;
        std::vector<int> TQ;
        for (int q = 0; q < 6; ++q) {   // two triangles per face: (o, u, u + v) and (o, u + v, v)
            const float* o = &Q[12 * q];
            const float* u = o + 3;
            const float* v = o + 6;
            for (int x = 0; x < 3; ++x) T.push_back(o[x]);
            for (int x = 0; x < 3; ++x) T.push_back(u[x]);
            for (int x = 0; x < 3; ++x) T.push_back(u[x] + v[x]);
            for (int x = 0; x < 3; ++x) T.push_back(o[x]);
            for (int x = 0; x < 3; ++x) T.push_back(u[x] + v[x]);
            for (int x = 0; x < 3; ++x) T.push_back(v[x]);
            TQ.push_back(q);
            TQ.push_back(q);
        }
        W(m.inten[si].data(), NLP * 4);
        W(P.data(), P.size() * 4);
        W(N.data(), N.size() * 4);
        W(Q, sizeof Q);
        W(dims.data(), dims.size() * 4);
        W(off.data(), off.size() * 4);
        W(T.data(), T.size() * 4);
        W(TQ.data(), TQ.size() * 4);
        if (with_ref) {
            W(m.ref[si].data(), (size_t)Np * 4);
            W(m.valid[si].data(), (size_t)Np);
            W(m.Pw[si].data(), (size_t)NLP * Np * 4);
        }
    }
    for (int a = 0; a < NS; ++a)
        for (int b = 0; b < NS; ++b) {
            std::vector<int> occ;
            if (a != b && m.boxpos[a] != m.boxpos[b]) {   // 12^3 samples of both cube positions
                for (int p = 0; p < 2; ++p)
                    for (int i = 0; i < 12; ++i)
                        for (int j = 0; j < 12; ++j)
                            for (int k = 0; k < 12; ++k) {
                                const float x[3] = {m.boxc[p][0] - m.boxe + 2 * m.boxe * i / 11.f, m.boxc[p][1] - m.boxe + 2 * m.boxe * j / 11.f,
                                                    m.boxc[p][2] - m.boxe + 2 * m.boxe * k / 11.f};
                                occ.push_back(host_vox(m, x));
                            }
                std::sort(occ.begin(), occ.end());
                occ.erase(std::unique(occ.begin(), occ.end()), occ.end());
            }
            const int no = (int)occ.size();
            W(&no, 4);
            W(occ.data(), occ.size() * 4);
            for (int l = 0; l < NLP; ++l) {
                std::vector<int> em;
                if (a != b && m.inten[a][l] == 0.f && m.inten[b][l] > 0.f) em.push_back(host_vox(m, &m.L[3 * l]));
                const int ne = (int)em.size();
                W(&ne, 4);
                W(em.data(), em.size() * 4);
            }
        }
    return out;
}

bool write_file(const char* path, const std::vector<uint8_t>& b) {
    FILE* f = fopen(path, "wb");
    if (!f) return false;
    const bool ok = fwrite(b.data(), 1, b.size(), f) == b.size();
    return fclose(f) == 0 && ok;
}

double since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

extern "C" rc_status rc_prep_mesh(rc_ctx* ctx, const char* mesh_path, const char* scene_path, int target, rc_prep_report* rep) {
    if (!ctx || !mesh_path || !scene_path || target < 16) return RC_ERR_ARG;
    const auto t0 = std::chrono::steady_clock::now();
    Mesh M;
    std::string err;
    if (!read_msh1(mesh_path, M, err)) return rc::ctx_fail(ctx, RC_ERR_IO, err.c_str());
    Prepared m;
    float hi[3];
    for (int a = 0; a < 3; ++a) { m.lo[a] = 1e30f; hi[a] = -1e30f; }
    for (size_t k = 0; k < M.V.size(); ++k) {
        const int a = (int)(k % 3);
        m.lo[a] = std::min(m.lo[a], M.V[k]);
        hi[a] = std::max(hi[a], M.V[k]);
    }
    const float diag = sqrtf((hi[0] - m.lo[0]) * (hi[0] - m.lo[0]) + (hi[1] - m.lo[1]) * (hi[1] - m.lo[1]) + (hi[2] - m.lo[2]) * (hi[2] - m.lo[2]));
    for (int a = 0; a < 3; ++a) {
        const float pad = 0.01f * diag + 0.05f;
        m.lo[a] -= pad;
        hi[a] += pad;
        m.ext[a] = hi[a] - m.lo[a];
    }
    // 1. BVH
    std::vector<int> order;
    build_bvh(M, m.BN, order);
    m.ST.resize(9 * (size_t)M.nt);
    m.STN.resize(4 * (size_t)M.nt);
    for (int j = 0; j < M.nt; ++j) {
        const float* v = &M.V[9 * (size_t)order[j]];
        float* T = &m.ST[9 * (size_t)j];
        for (int x = 0; x < 3; ++x) { T[x] = v[x]; T[3 + x] = v[3 + x] - v[x]; T[6 + x] = v[6 + x] - v[x]; }
        const float cr[3] = {T[4] * T[8] - T[5] * T[7], T[5] * T[6] - T[3] * T[8], T[3] * T[7] - T[4] * T[6]};
        float l = sqrtf(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
        l = l > 0 ? l : 1.f;
        const int fl = M.ds[order[j]] ? 1 : 0;
        for (int x = 0; x < 3; ++x) m.STN[4 * (size_t)j + x] = cr[x] / l;
        memcpy(&m.STN[4 * (size_t)j + 3], &fl, 4);
    }
    // 2. cache points: h aimed at the target count
    double atot = 0;
    for (int t = 0; t < M.nt; ++t) {
        const float* v = &M.V[9 * (size_t)t];
        const float e1[3] = {v[3] - v[0], v[4] - v[1], v[5] - v[2]}, e2[3] = {v[6] - v[0], v[7] - v[1], v[8] - v[2]};
        const float cr[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        atot += 0.5 * sqrt((double)cr[0] * cr[0] + (double)cr[1] * cr[1] + (double)cr[2] * cr[2]) * (M.ds[t] ? 2 : 1);
    }
    std::unordered_map<uint64_t, Cell> cells;
    m.h = (float)sqrt(atot / target);
    for (int it = 0; it < 5; ++it) {
        sample_cells(M, m.h, m.lo, cells);
        const double ratio = (double)cells.size() / target;
        if (fabs(ratio - 1.0) < 0.08 || it == 4) break;
        m.h *= (float)std::min(2.0, std::max(0.5, sqrt(ratio)));
    }
    std::vector<std::pair<uint64_t, uint64_t>> keys;   // (Morton order x 8 + bucket, key)
    keys.reserve(cells.size());
    for (auto& kv : cells) {
        int cx, cy, cz, b;
        key_cell(kv.first, cx, cy, cz, b);
        keys.push_back({(morton_spread(cx) | morton_spread(cy) << 1 | morton_spread(cz) << 2) * 8 + b, kv.first});
    }
    std::sort(keys.begin(), keys.end());
    m.npst = (int)keys.size();
    size_t HS = 1024;
    while (HS < 2 * (size_t)m.npst) HS <<= 1;
    m.HK.assign(HS, 0ull);
    m.HV.assign(HS, -1);
    std::unordered_map<uint64_t, int> zone;
    for (int i = 0; i < m.npst; ++i) {
        const Cell& c = cells[keys[i].second];
        for (int x = 0; x < 3; ++x) { m.Pst.push_back(c.p[x]); m.Nst.push_back(c.n[x]); }
        m.A.push_back((float)(c.wsum > 0 ? c.asum / c.wsum : 0.5));
        const uint64_t k = keys[i].second;
        size_t hh = (size_t)mix64(k) & (HS - 1);
        while (m.HK[hh] != 0ull) hh = (hh + 1) & (HS - 1);
        m.HK[hh] = k;
        m.HV[hh] = i;
        int cx, cy, cz, b;   // verification zone: 4 x 4 x 4 cells of one normal bucket
        key_cell(k, cx, cy, cz, b);
        auto z = zone.try_emplace(cell_key(cx >> 2, cy >> 2, cz >> 2, b), (int)zone.size());
        m.region.push_back(z.first->second);
    }
    cells.clear();
    m.NR = (int)zone.size();
    // 3. lamps and cube: free space from probe rays on the GPU
    const int NC = 16384;
    std::vector<float> C(3 * NC), O(3 * NC);
    {
        Rng r(12345);
        for (int i = 0; i < NC; ++i)
            for (int a = 0; a < 3; ++a) C[3 * i + a] = m.lo[a] + m.ext[a] * (0.03f + 0.94f * r.u());
    }
    {
        rc_status st = rc::ctx_probe_free_space(ctx, m.ST, m.STN, reinterpret_cast<const float*>(m.BN.data()), (int)m.BN.size(), C, diag, O);
        if (st != RC_OK) return st;
    }
    auto dist = [&](int a, const float* p) {
        float d = 0;
        for (int x = 0; x < 3; ++x) d += (C[3 * a + x] - p[x]) * (C[3 * a + x] - p[x]);
        return sqrtf(d);
    };
    std::vector<int> ok;
    float cmin = std::max(0.3f, 0.015f * diag), emin = 0.5f;
    for (int tries = 0; tries < 6 && ok.size() < 16; ++tries) {
        ok.clear();
        for (int i = 0; i < NC; ++i)
            if (O[3 * i] >= cmin && O[3 * i] < 1e29f && O[3 * i + 1] >= emin && O[3 * i + 2] <= 0.05f) ok.push_back(i);
        if (ok.size() < 16) { cmin *= 0.6f; emin = std::max(0.25f, emin - 0.1f); }
    }
    if (ok.size() < 3) return rc::ctx_fail(ctx, RC_ERR_FORMAT, "prep: not enough free space to place the lamps");
    std::vector<int> okL;   // lamps at 15 to 60 % of the scene's height
    for (int i : ok) {
        const float zr = (C[3 * i + 2] - m.lo[2]) / m.ext[2];
        if (zr >= 0.15f && zr <= 0.6f) okL.push_back(i);
    }
    if (okL.size() < 3) okL = ok;
    std::vector<int> Li;
    Li.push_back(*std::max_element(okL.begin(), okL.end(), [&](int a, int b) { return O[3 * a] < O[3 * b]; }));
    std::vector<float> cl;
    for (int i : okL) cl.push_back(O[3 * i]);
    std::nth_element(cl.begin(), cl.begin() + cl.size() / 2, cl.end());
    const float cmed = cl[cl.size() / 2];
    while ((int)Li.size() < NLP) {   // the clearest candidate farthest from the lamps placed so far
        int best = -1;
        float bd = -1;
        for (int i : okL) {
            if (O[3 * i] < cmed) continue;
            float d = 1e30f;
            for (int j : Li) d = std::min(d, dist(i, &C[3 * j]));
            if (d > bd) { bd = d; best = i; }
        }
        if (best < 0) return rc::ctx_fail(ctx, RC_ERR_FORMAT, "prep: no place for lamp %d", (int)Li.size());
        Li.push_back(best);
    }
    for (int j : Li)
        for (int x = 0; x < 3; ++x) m.L.push_back(C[3 * j + x]);
    float b = std::min(2.5f, std::max(0.25f, 0.06f * diag));
    int ia = -1, ib = -1;
    for (int tries = 0; tries < 8 && (ia < 0 || ib < 0); ++tries, b *= 0.75f) {
        ia = ib = -1;
        float da = 1e30f, db = 1e30f;
        auto clear_of_lamps = [&](int i) {
            for (int l = 0; l < NLP; ++l)
                if (dist(i, &m.L[3 * l]) < 1.2f * b) return false;
            return true;
        };
        for (int i : ok) {
            if (O[3 * i] < 1.0f * b || !clear_of_lamps(i)) continue;
            const float d0 = dist(i, &m.L[0]);
            if (d0 < da) { da = d0; ia = i; }
        }
        if (ia < 0) continue;
        for (int i : ok) {
            if (O[3 * i] < 1.0f * b || dist(i, &C[3 * ia]) < 2.f * b || !clear_of_lamps(i)) continue;
            const float d1 = dist(i, &m.L[3]);
            if (d1 < db) { db = d1; ib = i; }
        }
        if (ia >= 0 && ib >= 0) break;
    }
    if (ia < 0 || ib < 0) return rc::ctx_fail(ctx, RC_ERR_FORMAT, "prep: no place for the movable cube");
    m.boxe = 0.5f * b;
    for (int x = 0; x < 3; ++x) { m.boxc[0][x] = C[3 * ia + x]; m.boxc[1][x] = C[3 * ib + x]; }
    m.bnu = std::max(2, (int)std::lround(b / m.h));
    m.nbox = 6 * m.bnu * m.bnu;
    for (int k = 0; k < m.nbox; ++k) m.A.push_back(0.7f);
    {   // cube zones: 4 x 4 points per zone and face
        const int tu = (m.bnu + 3) / 4;
        for (int q = 0; q < 6; ++q)
            for (int iv = 0; iv < m.bnu; ++iv)
                for (int iu = 0; iu < m.bnu; ++iu) m.region.push_back(m.NR + q * tu * tu + (iv / 4) * tu + iu / 4);
        m.NR += 6 * tu * tu;
    }
    // 4. states: lamps 0, 1, 2 and the cube's position
    const float I[5][3] = {{1, 1, 0}, {0, 1, 0}, {1, 1, 0}, {1, 1, 1}, {0, 1, 0}};
    const int BP[5] = {0, 0, 1, 0, 1};
    for (int si = 0; si < 5; ++si) {
        m.inten.push_back(std::vector<float>(I[si], I[si] + 3));
        m.boxpos.push_back(BP[si]);
    }
    // 5. direct light normalised to a mean of 1 in state 0 (linear in the intensities)
    const int Np = m.npst + m.nbox;
    rc_status st;
    {
        std::vector<uint8_t> sb = scene_bytes(m, false);
        if ((st = rc_scene_load_memory(ctx, sb.data(), sb.size())) != RC_OK) return st;
        std::vector<float> Ed((size_t)NLP * Np);
        if ((st = rc_state_array_copy(ctx, 0, RC_SA_EDIR, Ed.data(), Ed.size() * 4)) != RC_OK) return st;
        double sm = 0;
        for (float x : Ed) sm += x;
        const float cn = sm > 0 ? (float)(Np / sm) : 1.f;
        for (auto& v : m.inten)
            for (auto& x : v) x *= cn;
        sb = scene_bytes(m, false);
        if ((st = rc_scene_load_memory(ctx, sb.data(), sb.size())) != RC_OK) return st;
    }
    // references (the preparation's parameters; PREP_BRUIT_CIBLE / PREP_ITER_MAX as there)
    rc_ref_params rp{32, 16, 64, 2048, 0.03};
    if (const char* e = getenv("PREP_BRUIT_CIBLE")) rp.noise_target = atof(e);
    if (const char* e = getenv("PREP_ITER_MAX")) rp.max_iter = std::max(rp.block, atoi(e));
    double noise[5];
    int iters[5];
    if ((st = rc_reference_build(ctx, &rp, noise, iters)) != RC_OK) return st;
    double vfrac = 0;
    for (int si = 0; si < 5; ++si) {
        std::vector<float> ref(Np), pw((size_t)NLP * Np);
        std::vector<uint8_t> val(Np);
        if ((st = rc_state_array_copy(ctx, si, RC_SA_REF, ref.data(), ref.size() * 4)) != RC_OK ||
            (st = rc_state_array_copy(ctx, si, RC_SA_VALID, val.data(), val.size())) != RC_OK ||
            (st = rc_state_array_copy(ctx, si, RC_SA_PW, pw.data(), pw.size() * 4)) != RC_OK)
            return st;
        long long nv = 0;
        for (uint8_t x : val) nv += x != 0;
        vfrac += (double)nv / Np / 5;
        m.ref.push_back(std::move(ref));
        m.valid.push_back(std::move(val));
        m.Pw.push_back(std::move(pw));
    }
    if (!write_file(scene_path, scene_bytes(m, true))) return rc::ctx_fail(ctx, RC_ERR_IO, "prep: cannot write %s", scene_path);
    if (rep) {
        memset(rep, 0, sizeof *rep);
        rep->triangles = M.nt;
        rep->np = Np;
        rep->zones = m.NR;
        rep->bvh_nodes = (int)m.BN.size();
        rep->cell_m = m.h;
        rep->diag_m = diag;
        rep->cube_m = b;
        rep->valid_fraction = vfrac;
        rep->ns = 5;
        for (int si = 0; si < 5; ++si) { rep->noise[si] = noise[si]; rep->iterations[si] = iters[si]; }
        for (int l = 0; l < NLP; ++l)
            for (int x = 0; x < 3; ++x) rep->lights[l][x] = m.L[3 * l + x];
        rep->seconds = since(t0);
    }
    return RC_OK;
}
