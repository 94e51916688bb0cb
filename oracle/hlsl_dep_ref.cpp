// The reference's bench dependency-marking shader functions (DepMarkPoint, DepMarkSegment of
// rtxgi_bench.patch:825-858, in the path tracer's SHaRC update pass) compiled as C++ on the CPU
// — TEST INFRASTRUCTURE ONLY.  oracle/build_hlsl_ref.sh extracts them unchanged from the
// reference checkout into oracle/_ref/hlsl_dep.inc (the only edit: HLSL's `inout` parameter
// becomes a C++ reference) and compiles this file with them, without contraction.  Used by
// tests/test_hlsl_pin.py to pin the restatement of those functions in oracle/hg_oracle.c.
#include "hlsl_compat.h"

#define DEP_GX 6
#define DEP_GY 4
#define DEP_GZ 4

#include "hlsl_dep.inc"

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
