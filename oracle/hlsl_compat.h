// HLSL vector types and intrinsics as plain C++ — TEST INFRASTRUCTURE ONLY.
//
// Just enough of HLSL's float3 / uint2 / uint3 / uint4 / bool3 arithmetic, of its intrinsics
// (any, all, min, max, abs, ceil, length, lerp, InterlockedAdd) and of its compute-shader
// resources to compile the bench's dependency-marking functions and snapshot shaders, taken
// from the reference's patch by oracle/build_patch_ref.sh, as C++ on the CPU.  Every operation is the IEEE single-precision one, component by component, in HLSL's
// definition order (lerp(x, y, s) = x + s * (y - x); length(v) = sqrt(dot(v, v)), the dot
// product summed x, y, z in that order); the recipe compiles without contraction.
#pragma once

#include <cmath>
#include <cstdint>

typedef uint32_t uint;

struct bool3 {
    bool x, y, z;
};
inline bool any(bool3 b) { return b.x || b.y || b.z; }
inline bool all(bool3 b) { return b.x && b.y && b.z; }

struct float3 {
    float x, y, z;
    float3() : x(0.f), y(0.f), z(0.f) {}
    float3(float a, float b, float c) : x(a), y(b), z(c) {}
};
inline float3 operator+(float3 a, float3 b) { return float3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline float3 operator-(float3 a, float3 b) { return float3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline float3 operator*(float3 a, float3 b) { return float3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline float3 operator/(float3 a, float3 b) { return float3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline float3 operator*(float3 a, float s) { return float3(a.x * s, a.y * s, a.z * s); }
inline float3 operator*(float s, float3 a) { return float3(s * a.x, s * a.y, s * a.z); }
inline bool3 operator<(float3 a, float s) { return {a.x < s, a.y < s, a.z < s}; }
inline bool3 operator>=(float3 a, float3 b) { return {a.x >= b.x, a.y >= b.y, a.z >= b.z}; }

struct uint3 {
    uint x, y, z;
    uint3() : x(0u), y(0u), z(0u) {}
    uint3(uint a, uint b, uint c) : x(a), y(b), z(c) {}
    explicit uint3(float3 f) : x((uint)f.x), y((uint)f.y), z((uint)f.z) {}   // truncation, as HLSL's conversion
};
struct uint2 {
    uint x, y;
};
struct uint4 {
    union {
        struct {
            uint x, y, z, w;
        };
        struct {
            uint2 xy, zw;
        };
    };
    uint4() : x(0u), y(0u), z(0u), w(0u) {}
    uint4(uint a, uint b, uint c, uint d) : x(a), y(b), z(c), w(d) {}
    uint4(uint2 a, uint c, uint d) : x(a.x), y(a.y), z(c), w(d) {}
};

// resources of a compute shader: a structured buffer is an array the harness points at, a
// constant buffer the struct itself; InterlockedAdd on one thread at a time (the harness runs
// the dispatch's threads in order)
template <class T>
struct RWStructuredBuffer {
    T* p = nullptr;
    T& operator[](uint i) const { return p[i]; }
};
template <class T>
using ConstantBuffer = T;
inline void InterlockedAdd(uint& dst, uint v) { dst += v; }
inline void InterlockedAdd(uint& dst, uint v, uint& original) {
    original = dst;
    dst += v;
}

inline float abs(float v) { return std::fabs(v); }
inline float min(float a, float b) { return std::fmin(a, b); }
inline float max(float a, float b) { return std::fmax(a, b); }
inline uint min(uint a, uint b) { return a < b ? a : b; }
inline float3 min(float3 a, float3 b) { return float3(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
inline float3 max(float3 a, float3 b) { return float3(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }
inline float ceil(float v) { return std::ceil(v); }
inline float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float length(float3 v) { return std::sqrt(dot(v, v)); }
inline float lerp(float x, float y, float s) { return x + s * (y - x); }

// the shader's constant buffer, as far as the marking functions read it
struct HlslFloat4 {
    float3 xyz;
    float w;
};
struct HlslGlobal {
    HlslFloat4 benchGridMin, benchGridMax;
};
static HlslGlobal g_Global;
