// common.cuh -- shared device helpers of the GB300 FD engine (sm_103a).
//
// Discretisation (jcottaar/seismic core/seis_forward2.py): 2nd order in time,
// 4th order in space, periodic wrap at the padded edge, sponge damping kappa =
// min_vel * damp(z,x) * dt, Ricker source at one padded point per shot.
//
// The reference advances p_{n+1} = temp1 p_n - temp2 p_{n-1} + alpha L'(p_n)
// with temp1 = 2 - 5 alpha - kappa, temp2 = 1 - kappa and L' the 12-point
// Laplacian without its centre (core/seis_forward2.py:333-344,381-462).  The
// kernels carry the same map in increment form, which keeps FP32 rounding an
// order of magnitude smaller over 1000-2000 steps:
//     u_{n+1} = (1 - kappa) u_n + alpha Lap(p_n) [+ s_mod at the source]
//     p_{n+1} = p_n + u_{n+1},         u_n = p_n - p_{n-1}
// where Lap(p) = L'(p) - 5p = c2 (sum of +-1 neighbours - 4p)
//                           + c3 (sum of +-2 neighbours - 4p).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace seis {

constexpr float kC2 = 4.0f / 3.0f;   // core/seis_forward2.py:80
constexpr float kC3 = -1.0f / 12.0f; // core/seis_forward2.py:81

// Padded-grid geometry as the kernels see it.  Fields are row-major with a
// row pitch of `pitch` floats (>= NX, multiple of 32); columns NX..pitch-1 are
// never read as wavefield values.
struct GridDev {
    int NZ, NX, pitch;
    int xlo, xhi;      // interior (non-sponge) columns [xlo, xhi) = [nbc, nbc+nx)
    int pad0;          // explicit, so that the struct has no implicit padding bytes
    long long NP;      // NZ * pitch
    int nt, nrec;
};
static_assert(sizeof(GridDev) == 40, "GridDev layout");

// Per concurrent shot slot of a chunk.
struct ShotDesc {
    int model;    // model index within the call
    int shot;     // shot index within the geometry
    int src_off;  // padded offset z*pitch + x of the source
    int active;   // 0 for slots past the last shot of the call
};

// damp(z,x) of AbcCoef2D (core/seis_forward2.py:46-59): the left/right bands
// cover every row (corners take the x profile), the top/bottom bands cover the
// interior columns only.  dampz is 0 on interior rows.
__device__ __forceinline__ float damp_at(int z, int x, const float* __restrict__ dampx,
                                         const float* __restrict__ dampz, const GridDev& g)
{
    return (x < g.xlo || x >= g.xhi) ? __ldg(dampx + x) : __ldg(dampz + z);
}

// Lap(p) at a point from its centre c and the neighbour sums t1 (+-1) and t2
// (+-2), with every rounding step spelled out so that the kernel variants that
// share it agree bitwise whatever the compiler would contract.
__device__ __forceinline__ float stencil_lap(float c, float t1, float t2)
{
    return __fmaf_rn(kC2, __fmaf_rn(-4.0f, c, t1), __fmul_rn(kC3, __fmaf_rn(-4.0f, c, t2)));
}
// 1 - kappa = 1 - (min_vel dt) damp, rounded as written (every kernel that
// forms it must agree bitwise: recomputed checkpoint segments and the cluster
// and tiled paths reuse each other's increments).
__device__ __forceinline__ float one_minus_kappa_of(float kf, float damp)
{
    return __fsub_rn(1.0f, __fmul_rn(kf, damp));
}
// u' = (1 - kappa) u + alpha Lap, rounded as written.
__device__ __forceinline__ float fwd_increment(float om, float u, float a, float lap)
{
    return __fmaf_rn(a, lap, __fmul_rn(om, u));
}

// Tangent increment du' = (1 - kappa) du + alpha Lap(dp) + alpha_d Lap(p) - kappa_d u,
// rounded as written (the linearisation of fwd_increment, prep_run_diff,
// core/seis_forward2.py:346-359,469-513).
__device__ __forceinline__ float tan_increment(float om, float du, float a, float dlap, float ad, float lap,
                                               float kd, float u)
{
    return __fsub_rn(__fmaf_rn(ad, lap, __fmaf_rn(a, dlap, __fmul_rn(om, du))), __fmul_rn(kd, u));
}

// The same arithmetic on a column pair at once: packed FP32 (f32x2) instructions,
// each lane rounded exactly as the scalar operation, so pair and single-column
// kernels agree bitwise.  Written as PTX with the explicit .rn modifier, which
// keeps the code generator from fusing a multiply and an add into one rounding.
__device__ __forceinline__ float2 splat2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b)
{
    float2 r;
    asm("{\n\t.reg .b64 pa, pb, pr;\n\tmov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
        "add.rn.f32x2 pr, pa, pb;\n\tmov.b64 {%0, %1}, pr;\n\t}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b)
{
    float2 r;
    asm("{\n\t.reg .b64 pa, pb, pr;\n\tmov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
        "mul.rn.f32x2 pr, pa, pb;\n\tmov.b64 {%0, %1}, pr;\n\t}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c)
{
    float2 r;
    asm("{\n\t.reg .b64 pa, pb, pc, pr;\n\tmov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
        "mov.b64 pc, {%6, %7};\n\tfma.rn.f32x2 pr, pa, pb, pc;\n\tmov.b64 {%0, %1}, pr;\n\t}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
    return r;
}
__device__ __forceinline__ float2 stencil_lap(float2 c, float2 t1, float2 t2)
{
    return fma2(splat2(kC2), fma2(splat2(-4.0f), c, t1), mul2(splat2(kC3), fma2(splat2(-4.0f), c, t2)));
}
__device__ __forceinline__ float2 fwd_increment(float2 om, float2 u, float2 a, float2 lap)
{
    return fma2(a, lap, mul2(om, u));
}
// The same with nkd = -kappa_d: x + (-kd) u rounds exactly as __fsub_rn(x, __fmul_rn(kd, u))
// (negation is exact and commutes with rounding to nearest).
__device__ __forceinline__ float tan_increment_nkd(float om, float du, float a, float dlap, float ad, float lap,
                                                   float nkd, float u)
{
    return __fadd_rn(__fmaf_rn(ad, lap, __fmaf_rn(a, dlap, __fmul_rn(om, du))), __fmul_rn(nkd, u));
}
// nkd = -kappa_d: x + (-kd) u rounds each lane exactly as __fsub_rn(x, __fmul_rn(kd, u))
// (negation is exact and commutes with rounding to nearest).
__device__ __forceinline__ float2 tan_increment_nkd(float2 om, float2 du, float2 a, float2 dlap, float2 ad,
                                                    float2 lap, float2 nkd, float2 u)
{
    return add2(fma2(ad, lap, fma2(a, dlap, mul2(om, du))), mul2(nkd, u));
}

__device__ __forceinline__ int wrap_idx(int i, int n)
{
    // every caller passes i >= -2; the modulo also keeps grids smaller than a tile correct
    return (i + 2 * n) % n;
}

}  // namespace seis
