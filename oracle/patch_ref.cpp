// Pieces of the reference's bench patch (windows/patch/rtxgi_bench.patch) compiled as C++ on the
// CPU — TEST INFRASTRUCTURE ONLY.  oracle/build_patch_ref.sh extracts them unchanged from a
// reference checkout into oracle/_ref/ and compiles this file with them, without contraction:
//   * DepMarkPoint, DepMarkSegment (patch:825-858, shader code of the path tracer's SHaRC update
//     pass; HLSL's `inout` parameter becomes a C++ reference), with HLSL's vector types from
//     oracle/hlsl_compat.h;
//   * Pathtracer::BenchObjVoxels (patch:592-615, host code: the event zones of an object), with a
//     stand-in for the members of the sample's Pathtracer class it reads;
//   * the snapshot compute shaders snapCount, snapPack, snapRestore of BenchSnap.hlsl
//     (patch:1283-1345), dispatched here one thread after another.
// Used by tests/test_patch_pin.py to pin oracle/hg_oracle.c and the library's rc_hg_event_mask.
#include <array>
#include <cstdint>
#include <vector>

#include "hlsl_compat.h"

#define DEP_GX 6
#define DEP_GY 4
#define DEP_GZ 4

#include "hlsl_dep.inc"

// what BenchObjVoxels reads of the sample's Pathtracer: the bench's zone box and its objects
// (objPos[i] = centre xyz and size xyz; a size of 0 takes the default half extent objHalf)
struct Pathtracer {
    struct {
        std::vector<std::array<float, 6>> objPos;
        float objHalf[3] = {0.f, 0.f, 0.f};
        float gridMin[3] = {0.f, 0.f, 0.f};
        float gridMax[3] = {0.f, 0.f, 0.f};
    } m_bench;
    void BenchObjVoxels(int obj, uint32_t inv[4]);
};

#include "bench_obj.inc"

#include "bench_snap.inc"

static void set_box(const float lo[3], const float hi[3]) {
    g_Global.benchGridMin.xyz = float3(lo[0], lo[1], lo[2]);
    g_Global.benchGridMax.xyz = float3(hi[0], hi[1], hi[2]);
}

extern "C" void href_mark_point(const float lo[3], const float hi[3], uint32_t m[3], const float p[3]) {
    set_box(lo, hi);
    uint3 mm(m[0], m[1], m[2]);
    DepMarkPoint(mm, float3(p[0], p[1], p[2]));
    m[0] = mm.x;
    m[1] = mm.y;
    m[2] = mm.z;
}

extern "C" void href_mark_segment(const float lo[3], const float hi[3], uint32_t m[3], const float a[3], const float b[3]) {
    set_box(lo, hi);
    uint3 mm(m[0], m[1], m[2]);
    DepMarkSegment(mm, float3(a[0], a[1], a[2]), float3(b[0], b[1], b[2]));
    m[0] = mm.x;
    m[1] = mm.y;
    m[2] = mm.z;
}

// the zones of one object (centre xyz, size xyz) or-ed into inv[0..2]
extern "C" void href_obj_voxels(const float lo[3], const float hi[3], const float obj[6], uint32_t inv[4]) {
    Pathtracer pt;
    for (int k = 0; k < 3; ++k) {
        pt.m_bench.gridMin[k] = lo[k];
        pt.m_bench.gridMax[k] = hi[k];
    }
    pt.m_bench.objPos.push_back({obj[0], obj[1], obj[2], obj[3], obj[4], obj[5]});
    pt.BenchObjVoxels(0, inv);
}

// snapCount then snapPack over a table of `cap` entries (keys as the shader's uint2: low word,
// high word; resolved as uint4), records into `recs` (at most rec_cap); returns the count
extern "C" uint32_t href_snapshot(uint64_t* keys, uint32_t* resolved, uint32_t cap, void* recs, uint32_t rec_cap) {
    static_assert(sizeof(SnapRec) == 24 && sizeof(uint4) == 16 && sizeof(uint2) == 8, "record layout");
    uint counter = 0;
    u_Hash.p = reinterpret_cast<uint2*>(keys);
    u_Resolved.p = reinterpret_cast<uint4*>(resolved);
    u_Snap.p = reinterpret_cast<SnapRec*>(recs);
    u_Counter.p = &counter;
    g_Snap.capacity = cap;
    g_Snap.count = rec_cap;
    for (uint id = 0; id < cap; ++id) snapCount(id);
    const uint n = counter;
    counter = 0;
    for (uint id = 0; id < cap; ++id) snapPack(id);
    return n;
}

// snapRestore of `count` records into the table
extern "C" void href_restore(uint64_t* keys, uint32_t* resolved, uint32_t cap, void* recs, uint32_t count) {
    u_Hash.p = reinterpret_cast<uint2*>(keys);
    u_Resolved.p = reinterpret_cast<uint4*>(resolved);
    u_Snap.p = reinterpret_cast<SnapRec*>(recs);
    g_Snap.capacity = cap;
    g_Snap.count = count;
    for (uint id = 0; id < count; ++id) snapRestore(id);
}
