// sweep_kernels.cuh -- tiled per-time-step sweep kernels (any grid size).
//
// One launch advances every shot slot of a chunk by one time step
// (grid = tiles_x x tiles_z x shot slots); a sweep of nt launches is captured
// once in a CUDA graph and replayed, as the reference does per shot
// (core/seis_forward2.py:211-246).  The wavefields live in global memory (L2
// for moderate chunks); each block stages its 32x16 tile plus a 2-cell halo
// in shared memory and applies the stencil from there.
//
// Forward (+ tangent) step, reference kernels lapg + update_p (+ update_p_diff),
// core/seis_forward2.py:381-513, in the increment form of common.cuh:
//   u'  = (1-k) u + a Lap(p) + s_mod[t] d_src           p'  = p + u'
//   du' = (1-k) du + a Lap(dp) + ad Lap(p) - kd u + s_mod_diff[t] d_src
//                                                       dp' = dp + du'
// with a = alpha, k = kappa, ad / kd their derivatives along vec_diff
// (prep_run_diff, core/seis_forward2.py:346-359).
//
// Adjoint step, reference kernel update_p_adjoint (core/seis_forward2.py:516-579).
// With lambda_j = dJ/dp_j the reference recursion is
//   lambda_j = seed_j + temp1 lambda_{j+1} + L'(alpha lambda_{j+1}) - temp2 lambda_{j+2},
// which in increment form (mu_j = lambda_j - lambda_{j+1}) reads
//   mu_j = seed_j + (1-k) mu_{j+1} + Lap(alpha lambda_{j+1}),  lambda_j = lambda_{j+1} + mu_j.
// The coefficient gradients the reference accumulates per step
// (temp1/temp2/alpha adjoints, :549-553) and folds in prep_run_adjoint
// (:361-377) collapse to two per-point sums over t:
//   Gv = sum_t lambda_{t+2} (u_{t+2} - (1-k) u_{t+1})   [= alpha Lap(p_{t+1}) + s_mod d_src]
//   Gk = sum_t lambda_{t+2} u_{t+1}
// giving dJ/dv = (2/v) Gv (the explicit source-term gradient of :314 cancels
// against the source part of u) and dJ/dmin_vel = -dt sum_x damp Gk.  The
// forward sweep therefore stores only u (one FP32 level per step).
#pragma once
#include "common.cuh"

namespace seis {
// Kernels have internal linkage so that every translation unit that includes
// this header gets its own copy (no relocatable device code is used).
namespace {

// Tile of one block: kTX columns x kTZ rows; block kBX x kBZ threads, each
// thread a column pair (8-byte accesses) on kTZ / kBZ rows spaced kBZ apart,
// so that a warp covers one row of the tile (coalesced 256-byte accesses).
constexpr int kTX = 64;           // tile columns
constexpr int kTZ = 32;           // tile rows
constexpr int kBX = 32;           // block columns of threads (one warp)
constexpr int kBZ = 8;            // block rows of threads
constexpr int kRPTile = kTZ / kBZ;  // rows per thread
constexpr int kThreads = kBX * kBZ;
constexpr int kSW = kTX + 4;      // staged tile width with the 2-cell halo (even: 8-byte aligned pairs)
constexpr int kSH = kTZ + 4;

struct FwdArgs {
    GridDev g;
    const ShotDesc* shots;
    const float* alpha;      // [model][NP]
    const float* kfac;       // [model] min_vel*dt
    const float* alpha_d;    // [model][NP]   (tangent)
    const float* kdfac;      // [model] min_vel_diff*dt (tangent)
    const float* dampx;      // [pitch]
    const float* dampz;      // [NZ]
    float* p;                // [slot][3][NP]: p_m in level m % 3
    float* u;                // [slot][ulevels][NP]
    long long u_slot_stride;
    int ulevels;             // 3 (ring) or nt+1 (history kept for the adjoint)
    int pad0;                // explicit padding (the wavefront sweeps compare these structs bytewise)
    float* dp;               // [slot][3][NP]  (tangent): dp_m in level m % 3
    float* du;               // [slot][3][NP]  (tangent): du_m in level (m-1) % 3
    const float* smod;       // [slot][nt]
    const float* smod_d;     // [slot][nt]    (tangent)
    float* rec;              // [slot][nt][nrec]
    float* drec;             // [slot][nt][nrec] (tangent)
    const int* tile_rec_start;  // [tiles+1]
    const int* tile_rec_list;   // receiver ids grouped by tile
    const int* rec_off;         // [nrec] padded offsets
};

struct AdjArgs {
    GridDev g;
    const ShotDesc* shots;
    const float* alpha;
    const float* kfac;
    const float* dampx;
    const float* dampz;
    const float* u;          // [slot][ulevels][NP] forward increments, level l = u_{l+1} at l % ulevels
    long long u_slot_stride;
    int ulevels;             // nt+1 (whole history) or k+1 (ring of a recomputed checkpoint segment)
    int pad0;
    float* lam;              // [slot][3][NP]: lambda_m in level m % 3
    float* mu;               // [slot][3][NP]: mu_m in level m % 3
    float* gv;               // [slot][NP]
    float* gk;               // [slot][NP]
    const float* seed;       // [slot][nt][nrec]
    const int* tile_rec_start;
    const int* tile_rec_list;
    const int* rec_off;
};

static_assert(sizeof(FwdArgs) == 200 && sizeof(AdjArgs) == 168, "argument structs without implicit padding");

// Periodic index of a staged row / column (offset -2 .. n+tile): one conditional
// wrap when the grid is at least a staged tile wide, else the general modulo.
__device__ __forceinline__ int wrap_staged(int i, int n, bool small)
{
    if (small) return wrap_idx(i, n);
    return i < 0 ? i + n : (i >= n ? i - n : i);
}

// Stage the tile of f (plus its 2-cell halo, periodic) in shared memory,
// optionally multiplied point by point by w (the adjoint's alpha * lambda).
template <bool MUL>
__device__ __forceinline__ void stage_tile(float (*s)[kSW], const float* __restrict__ f,
                                           const float* __restrict__ w, int z0, int x0, const GridDev& g)
{
    const bool small = g.NX < kSW || g.NZ < kSH;
    // each thread stages one pair of columns (kTX/2 pairs + 2 halo pairs) of rows ty, ty + kBZ, ...
    const bool pairs = !small && (g.NX % 2 == 0);
    for (int j = threadIdx.y; j < kSH; j += kBZ) {
        const long long rowo = (long long)wrap_staged(z0 - 2 + j, g.NZ, small) * g.pitch;
        for (int q = threadIdx.x; q < kSW / 2; q += kBX) {
            const int i = 2 * q;
            if (pairs) {
                // NX even: a pair never straddles the wrap (x0 is even)
                const long long o = rowo + wrap_staged(x0 - 2 + i, g.NX, false);
                float2 v = *reinterpret_cast<const float2*>(f + o);
                if (MUL) {
                    const float2 c = __ldg(reinterpret_cast<const float2*>(w + o));
                    v.x = __fmul_rn(c.x, v.x);
                    v.y = __fmul_rn(c.y, v.y);
                }
                *reinterpret_cast<float2*>(&s[j][i]) = v;
            } else {
#pragma unroll
                for (int e = 0; e < 2; ++e) {
                    const long long o = rowo + wrap_staged(x0 - 2 + i + e, g.NX, small);
                    s[j][i + e] = MUL ? __fmul_rn(__ldg(w + o), f[o]) : f[o];
                }
            }
        }
    }
}

// Lap at the pair of tile-local columns (xx, xx+1) of staged row zz (halo
// offset included), in the sum order of the cluster kernels' downward walk.
template <int SW = kSW>
__device__ __forceinline__ float2 lap_pair(const float (*s)[SW], int zz, int xx, float2& c)
{
    c = *reinterpret_cast<const float2*>(&s[zz][xx]);
    const float2 l = *reinterpret_cast<const float2*>(&s[zz][xx - 2]);
    const float2 r = *reinterpret_cast<const float2*>(&s[zz][xx + 2]);
    const float2 n1 = *reinterpret_cast<const float2*>(&s[zz - 1][xx]);
    const float2 s1 = *reinterpret_cast<const float2*>(&s[zz + 1][xx]);
    const float2 n2 = *reinterpret_cast<const float2*>(&s[zz - 2][xx]);
    const float2 s2 = *reinterpret_cast<const float2*>(&s[zz + 2][xx]);
    // column xx: east c.y, west l.y, east2 r.x, west2 l.x; column xx+1: east r.x, west c.x, east2 r.y, west2 l.y;
    // both columns at once in packed FP32, each lane rounded as the scalar sums
    const float2 t1 = add2(make_float2(c.y + l.y, r.x + c.x), add2(s1, n1));
    const float2 t2 = add2(add2(r, l), add2(s2, n2));
    return stencil_lap(c, t1, t2);
}

// 1 - kappa of (z, x): side bands by column, elsewhere by row (AbcCoef2D).
__device__ __forceinline__ float one_minus_kappa(float kf, int z, int x, const float* __restrict__ dampx,
                                                 const float* __restrict__ dampz, const GridDev& g)
{
    return one_minus_kappa_of(kf, damp_at(z, x, dampx, dampz, g));
}

// One forward step t of tile (bx, by) of slot `slot` (tiles_x tiles per row), staged
// in sp (and sdp for the tangent): the body of fwd_step_kernel, also run as one item
// of the persistent wavefront sweeps.
template <bool TAN>
__device__ __forceinline__ void fwd_step_tile(const FwdArgs& a, int t, int slot, int bx, int by, int tiles_x,
                                              float (*sp)[kSW], float (*sdp)[kSW])
{
    const ShotDesc sd = a.shots[slot];
    if (!sd.active) return;
    const GridDev& g = a.g;
    const int x0 = bx * kTX, z0 = by * kTZ;
    const long long NP = g.NP;

    const float* pcur = a.p + (long long)slot * 3 * NP + (long long)((t + 1) % 3) * NP;   // p_{t+1}
    float* pnext = a.p + (long long)slot * 3 * NP + (long long)((t + 2) % 3) * NP;        // p_{t+2}
    const float* ucur = a.u + (long long)slot * a.u_slot_stride + (long long)(t % a.ulevels) * NP;
    float* unext = a.u + (long long)slot * a.u_slot_stride + (long long)((t + 1) % a.ulevels) * NP;
    const float* dpcur = nullptr;
    float* dpnext = nullptr;
    const float* ducur = nullptr;
    float* dunext = nullptr;
    if (TAN) {
        dpcur = a.dp + (long long)slot * 3 * NP + (long long)((t + 1) % 3) * NP;   // dp_{t+1}
        dpnext = a.dp + (long long)slot * 3 * NP + (long long)((t + 2) % 3) * NP;  // dp_{t+2}
        ducur = a.du + (long long)slot * 3 * NP + (long long)(t % 3) * NP;         // du_{t+1}
        dunext = a.du + (long long)slot * 3 * NP + (long long)((t + 1) % 3) * NP;  // du_{t+2}
    }
    stage_tile<false>(sp, pcur, nullptr, z0, x0, g);
    if (TAN) stage_tile<false>(sdp, dpcur, nullptr, z0, x0, g);
    __syncthreads();

    const float* al = a.alpha + (long long)sd.model * NP;
    const float kf = __ldg(a.kfac + sd.model);
    const float* ald = TAN ? a.alpha_d + (long long)sd.model * NP : nullptr;
    const float kdf = TAN ? __ldg(a.kdfac + sd.model) : 0.0f;
    const float src = __ldg(a.smod + (long long)slot * g.nt + t);
    const float src_d = TAN ? __ldg(a.smod_d + (long long)slot * g.nt + t) : 0.0f;
    const int xx = 2 * threadIdx.x;          // tile-local first column of the pair
    const int x = x0 + xx;
    const bool v0 = x < g.NX, v1 = x + 1 < g.NX;
#pragma unroll
    for (int r = 0; r < kRPTile; ++r) {
        const int zz = threadIdx.y + r * kBZ;
        const int z = z0 + zz;
        if (!v0 || z >= g.NZ) continue;
        const int i = z * g.pitch + x;       // offset within a field (< 2^31)
        float2 c;
        const float2 L = lap_pair(sp, zz + 2, xx + 2, c);
        const float2 aa = __ldg(reinterpret_cast<const float2*>(al + i));
        const float2 uc = *reinterpret_cast<const float2*>(ucur + i);
        const float om0 = one_minus_kappa(kf, z, x, a.dampx, a.dampz, g);
        const float om1 = v1 ? one_minus_kappa(kf, z, x + 1, a.dampx, a.dampz, g) : 0.0f;
        const float2 un = fwd_increment(make_float2(om0, om1), uc, aa, L);
        float un0 = un.x, un1 = un.y;
        if (i == sd.src_off) un0 += src;
        if (i + 1 == sd.src_off) un1 += src;
        float dun0 = 0.0f, dun1 = 0.0f;
        float2 dc;
        if (TAN) {
            const float2 dL = lap_pair(sdp, zz + 2, xx + 2, dc);
            const float2 ad = __ldg(reinterpret_cast<const float2*>(ald + i));
            const float2 du = *reinterpret_cast<const float2*>(ducur + i);
            const float kd0 = __fmul_rn(kdf, damp_at(z, x, a.dampx, a.dampz, g));
            const float kd1 = v1 ? __fmul_rn(kdf, damp_at(z, x + 1, a.dampx, a.dampz, g)) : 0.0f;
            dun0 = tan_increment(om0, du.x, aa.x, dL.x, ad.x, L.x, kd0, uc.x);
            dun1 = tan_increment(om1, du.y, aa.y, dL.y, ad.y, L.y, kd1, uc.y);
            if (i == sd.src_off) dun0 += src_d;
            if (i + 1 == sd.src_off) dun1 += src_d;
        }
        if (v1) {
            *reinterpret_cast<float2*>(unext + i) = make_float2(un0, un1);
            *reinterpret_cast<float2*>(pnext + i) = make_float2(c.x + un0, c.y + un1);
            if (TAN) {
                *reinterpret_cast<float2*>(dunext + i) = make_float2(dun0, dun1);
                *reinterpret_cast<float2*>(dpnext + i) = make_float2(dc.x + dun0, dc.y + dun1);
            }
        } else {
            unext[i] = un0;
            pnext[i] = c.x + un0;
            if (TAN) {
                dunext[i] = dun0;
                dpnext[i] = dc.x + dun0;
            }
        }
    }
    // receiver gather of this tile (record row t = level t+2, core/seis_forward2.py:249)
    const int tile = by * tiles_x + bx;
    const int r0 = a.tile_rec_start[tile], r1 = a.tile_rec_start[tile + 1];
    if (r1 > r0) {
        __syncthreads();
        const int tid = threadIdx.y * kBX + threadIdx.x;
        for (int k = r0 + tid; k < r1; k += kThreads) {
            const int rr = a.tile_rec_list[k];
            const long long o = ((long long)slot * g.nt + t) * g.nrec + rr;
            a.rec[o] = pnext[a.rec_off[rr]];
            if (TAN) a.drec[o] = dpnext[a.rec_off[rr]];
        }
    }
}

template <bool TAN>
__global__ void __launch_bounds__(kThreads) fwd_step_kernel(FwdArgs a, int t)
{
    __shared__ __align__(16) float sp[kSH][kSW];
    __shared__ __align__(16) float sdp[TAN ? kSH : 1][kSW];
    fwd_step_tile<TAN>(a, t, blockIdx.z, blockIdx.x, blockIdx.y, gridDim.x, sp, sdp);
}

// Reverse step t (t = nt-1 .. 0): lambda_{t+2} from lambda_{t+3}, mu_{t+3};
// the same rounding as the cluster adjoint (stencil_lap and fused multiply-adds
// spelled out), so both paths give bitwise the same gradients.
__device__ __forceinline__ void adj_step_tile(const AdjArgs& a, int t, int slot, int bx, int by, int tiles_x,
                                              float (*sm)[kSW], float (*sseed)[kTX])
{
    const ShotDesc sd = a.shots[slot];
    if (!sd.active) return;
    const GridDev& g = a.g;
    const int x0 = bx * kTX, z0 = by * kTZ;
    const long long NP = g.NP;
    const float* lprev = a.lam + (long long)slot * 3 * NP + (long long)(t % 3) * NP;        // lambda_{t+3}
    float* lnext = a.lam + (long long)slot * 3 * NP + (long long)((t + 2) % 3) * NP;       // lambda_{t+2}
    const float* al = a.alpha + (long long)sd.model * NP;
    const int tid = threadIdx.y * kBX + threadIdx.x;

    stage_tile<true>(sm, lprev, al, z0, x0, g);     // alpha * lambda_{t+3}
    const int tile = by * tiles_x + bx;
    const int r0 = a.tile_rec_start[tile], r1 = a.tile_rec_start[tile + 1];
    const bool has_rec = r1 > r0;
    if (has_rec) {
        for (int k = tid; k < kTZ * kTX; k += kThreads) (&sseed[0][0])[k] = 0.0f;
        __syncthreads();
        for (int k = r0 + tid; k < r1; k += kThreads) {
            const int rr = a.tile_rec_list[k];
            const int off = a.rec_off[rr];
            const int rz = off / g.pitch - z0, rx = off % g.pitch - x0;
            sseed[rz][rx] = a.seed[((long long)slot * g.nt + t) * g.nrec + rr];
        }
    }
    __syncthreads();

    const float kf = __ldg(a.kfac + sd.model);
    const float* u2 = a.u + (long long)slot * a.u_slot_stride + (long long)((t + 1) % a.ulevels) * NP;  // u_{t+2}
    const float* u1 = a.u + (long long)slot * a.u_slot_stride + (long long)(t % a.ulevels) * NP;        // u_{t+1}
    const float* mu = a.mu + (long long)slot * 3 * NP + (long long)(t % 3) * NP;          // mu_{t+3}
    float* munext = a.mu + (long long)slot * 3 * NP + (long long)((t + 2) % 3) * NP;      // mu_{t+2}
    float* gv = a.gv + (long long)slot * NP;
    float* gk = a.gk + (long long)slot * NP;
    const int xx = 2 * threadIdx.x;
    const int x = x0 + xx;
    const bool v0 = x < g.NX, v1 = x + 1 < g.NX;
#pragma unroll
    for (int r = 0; r < kRPTile; ++r) {
        const int zz = threadIdx.y + r * kBZ;
        const int z = z0 + zz;
        if (!v0 || z >= g.NZ) continue;
        const int i = z * g.pitch + x;
        float2 cdummy;
        const float2 Lm = lap_pair(sm, zz + 2, xx + 2, cdummy);
        const float om0 = one_minus_kappa(kf, z, x, a.dampx, a.dampz, g);
        const float om1 = v1 ? one_minus_kappa(kf, z, x + 1, a.dampx, a.dampz, g) : 0.0f;
        const float2 m0 = *reinterpret_cast<const float2*>(mu + i);
        const float2 lp = *reinterpret_cast<const float2*>(lprev + i);
        const float2 a1 = *reinterpret_cast<const float2*>(u1 + i);
        const float2 a2 = *reinterpret_cast<const float2*>(u2 + i);
        float2 gvv = *reinterpret_cast<const float2*>(gv + i);
        float2 gkk = *reinterpret_cast<const float2*>(gk + i);
        const float2 mm = fma2(make_float2(om0, om1), m0, Lm);
        float m_0 = mm.x, m_1 = mm.y;
        if (has_rec) {
            m_0 += sseed[zz][xx];
            m_1 += sseed[zz][xx + 1];
        }
        const float2 ll = add2(lp, make_float2(m_0, m_1));
        const float l0 = ll.x, l1 = ll.y;
        gvv = fma2(ll, fma2(make_float2(-om0, -om1), a1, a2), gvv);
        gkk = fma2(ll, a1, gkk);
        if (v1) {
            *reinterpret_cast<float2*>(munext + i) = make_float2(m_0, m_1);
            *reinterpret_cast<float2*>(lnext + i) = make_float2(l0, l1);
            *reinterpret_cast<float2*>(gv + i) = gvv;
            *reinterpret_cast<float2*>(gk + i) = gkk;
        } else {
            munext[i] = m_0;
            lnext[i] = l0;
            gv[i] = gvv.x;
            gk[i] = gkk.x;
        }
    }
}

__global__ void __launch_bounds__(kThreads) adj_step_kernel(AdjArgs a, int t)
{
    __shared__ __align__(16) float sm[kSH][kSW];
    __shared__ __align__(16) float sseed[kTZ][kTX];
    adj_step_tile(a, t, blockIdx.z, blockIdx.x, blockIdx.y, gridDim.x, sm, sseed);
}

// ---------------------------------------------------------------------------
// Two reverse steps t and t-1 in one launch (t >= 1; even NX at least kFW wide
// and kFH tall).  The block stages alpha * lambda_{t+3} on its tile plus a
// 4-cell halo, computes step t on the tile plus a 2-cell halo in shared memory
// (lambda_{t+2}, mu_{t+2} and alpha * lambda_{t+2} there), then step t-1 on the
// tile, and reads / writes lambda, mu and the gradient sums once for both steps.
// Every point gets the arithmetic of adj_step_kernel in the same order, so the
// results are bitwise those of two single steps (and of the cluster adjoint).
// lambda_{t+3} and alpha are staged raw by asynchronous copies (all in flight at once)
// and multiplied in shared memory.  Dynamic shared memory: kFusedAdjSmem bytes.
constexpr int kFW = kTX + 8, kFH = kTZ + 8;    // staged width / height with the 4-cell halo
constexpr int kFusedAdjSmem = 4 * (2 * kFH * kFW + 2 * kSH * kSW);
constexpr int kFusedTasks = (kSH * (kSW / 2) + kThreads - 1) / kThreads;   // step-t pairs per thread

__device__ __forceinline__ int wrap_once(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

// 8-byte asynchronous copy global -> shared (both 8-byte aligned), completed by
// async_copies_wait(): the staging loads of a tile all in flight at once, without
// passing through registers.
__device__ __forceinline__ void async_copy8(void* smem_dst, const void* gsrc)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void async_copies_wait()
{
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

// Two forward steps t and t+1 in one launch (same conditions as the fused adjoint):
// p_{t+1} (and the tangent's dp_{t+1}) staged with a 4-cell halo, step t on the tile
// plus a 2-cell halo in shared memory (p_{t+2}, u_{t+2}; dp_{t+2}, du_{t+2}), step t+1
// on the tile; u, du, alpha and dalpha read once for both steps.  Bitwise two single
// steps.
template <bool TAN>
constexpr int fused_fwd_smem() { return 4 * ((TAN ? 2 : 1) * kFH * kFW + (TAN ? 4 : 2) * kSH * kSW); }

template <bool TAN>
__device__ __forceinline__ void fwd_step2_tile(const FwdArgs& a, int t, int slot, int bx, int by, int tiles_x,
                                               float* fsm)
{
    float (*sP)[kFW] = reinterpret_cast<float (*)[kFW]>(fsm);                     // p_{t+1}, halo 4
    float (*sDP)[kFW] = sP + kFH;                                                 // dp_{t+1}, halo 4 (TAN)
    float (*sQ)[kSW] = reinterpret_cast<float (*)[kSW]>(fsm + (TAN ? 2 : 1) * kFH * kFW);   // p_{t+2}, halo 2
    float (*sU)[kSW] = sQ + kSH;                                                  // u_{t+2}, halo 2
    float (*sDQ)[kSW] = sU + kSH;                                                 // dp_{t+2} (TAN)
    float (*sDU)[kSW] = sDQ + kSH;                                                // du_{t+2} (TAN)
    const ShotDesc sd = a.shots[slot];
    if (!sd.active) return;
    const GridDev& g = a.g;
    const int x0 = bx * kTX, z0 = by * kTZ;
    const long long NP = g.NP;
    const int tid = threadIdx.y * kBX + threadIdx.x;
    const long long ps = (long long)slot * 3 * NP;
    const float* p1 = a.p + ps + (long long)((t + 1) % 3) * NP;        // p_{t+1}
    float* p3 = a.p + ps + (long long)(t % 3) * NP;                    // p_{t+3}
    const float* u1 = a.u + (long long)slot * a.u_slot_stride + (long long)(t % a.ulevels) * NP;          // u_{t+1}
    float* u2 = a.u + (long long)slot * a.u_slot_stride + (long long)((t + 1) % a.ulevels) * NP;          // u_{t+2}
    float* u3 = a.u + (long long)slot * a.u_slot_stride + (long long)((t + 2) % a.ulevels) * NP;          // u_{t+3}
    const float* dp1 = TAN ? a.dp + ps + (long long)((t + 1) % 3) * NP : nullptr;   // dp_{t+1}
    float* dp3 = TAN ? a.dp + ps + (long long)(t % 3) * NP : nullptr;               // dp_{t+3}
    const float* du1 = TAN ? a.du + ps + (long long)(t % 3) * NP : nullptr;         // du_{t+1}
    float* du2 = TAN ? a.du + ps + (long long)((t + 1) % 3) * NP : nullptr;         // du_{t+2}
    float* du3 = TAN ? a.du + ps + (long long)((t + 2) % 3) * NP : nullptr;         // du_{t+3}
    const float* al = a.alpha + (long long)sd.model * NP;
    const float* ald = TAN ? a.alpha_d + (long long)sd.model * NP : nullptr;
    const float kf = __ldg(a.kfac + sd.model);
    const float kdf = TAN ? __ldg(a.kdfac + sd.model) : 0.0f;
    const float src = __ldg(a.smod + (long long)slot * g.nt + t);
    const float src2 = __ldg(a.smod + (long long)slot * g.nt + t + 1);
    const float srcd = TAN ? __ldg(a.smod_d + (long long)slot * g.nt + t) : 0.0f;
    const float srcd2 = TAN ? __ldg(a.smod_d + (long long)slot * g.nt + t + 1) : 0.0f;

    // this thread's step-t pairs (tile + halo 2): u_{t+1} and alpha loads issued up front
    float2 uu[kFusedTasks], av[kFusedTasks];
#pragma unroll
    for (int it = 0; it < kFusedTasks; ++it) {
        const int k = tid + it * kThreads;
        uu[it] = av[it] = make_float2(0.0f, 0.0f);
        if (k < kSH * (kSW / 2)) {
            const int j = k / (kSW / 2), i = 2 * (k - j * (kSW / 2));
            const long long o = (long long)wrap_once(z0 - 2 + j, g.NZ) * g.pitch + wrap_once(x0 - 2 + i, g.NX);
            uu[it] = *reinterpret_cast<const float2*>(u1 + o);
            av[it] = __ldg(reinterpret_cast<const float2*>(al + o));
        }
    }
#pragma unroll
    for (int j = threadIdx.y; j < kFH; j += kBZ) {
        const long long rowo = (long long)wrap_once(z0 - 4 + j, g.NZ) * g.pitch;
#pragma unroll
        for (int q = threadIdx.x; q < kFW / 2; q += kBX) {
            const long long o = rowo + wrap_once(x0 - 4 + 2 * q, g.NX);
            async_copy8(&sP[j][2 * q], p1 + o);
            if (TAN) async_copy8(&sDP[j][2 * q], dp1 + o);
        }
    }
    async_copies_wait();
    __syncthreads();

    // step t on the tile + halo 2; u_{t+2} (du_{t+2}) of the tile's own points to its level
#pragma unroll
    for (int it = 0; it < kFusedTasks; ++it) {
        const int k = tid + it * kThreads;
        if (k >= kSH * (kSW / 2)) break;
        const int j = k / (kSW / 2), i = 2 * (k - j * (kSW / 2));
        const int z = wrap_once(z0 - 2 + j, g.NZ), x = wrap_once(x0 - 2 + i, g.NX);
        float2 c;
        const float2 L = lap_pair<kFW>(sP, j + 2, i + 2, c);
        const float om0 = one_minus_kappa(kf, z, x, a.dampx, a.dampz, g);
        const float om1 = one_minus_kappa(kf, z, x + 1, a.dampx, a.dampz, g);
        const float2 un = fwd_increment(make_float2(om0, om1), uu[it], av[it], L);
        float un0 = un.x, un1 = un.y;
        const int o = z * g.pitch + x;
        if (o == sd.src_off) un0 += src;
        if (o + 1 == sd.src_off) un1 += src;
        const float2 un2 = make_float2(un0, un1);
        *reinterpret_cast<float2*>(&sU[j][i]) = un2;
        *reinterpret_cast<float2*>(&sQ[j][i]) = add2(c, un2);
        const bool own = j >= 2 && j < kTZ + 2 && i >= 2 && i < kTX + 2 && z0 + j - 2 < g.NZ && x0 + i - 2 < g.NX;
        if (own) *reinterpret_cast<float2*>(u2 + o) = make_float2(un0, un1);
        if (TAN) {
            float2 dc;
            const float2 dL = lap_pair<kFW>(sDP, j + 2, i + 2, dc);
            const float2 ad = __ldg(reinterpret_cast<const float2*>(ald + o));
            const float2 du = *reinterpret_cast<const float2*>(du1 + o);
            const float kd0 = __fmul_rn(kdf, damp_at(z, x, a.dampx, a.dampz, g));
            const float kd1 = __fmul_rn(kdf, damp_at(z, x + 1, a.dampx, a.dampz, g));
            float dun0 = tan_increment(om0, du.x, av[it].x, dL.x, ad.x, L.x, kd0, uu[it].x);
            float dun1 = tan_increment(om1, du.y, av[it].y, dL.y, ad.y, L.y, kd1, uu[it].y);
            if (o == sd.src_off) dun0 += srcd;
            if (o + 1 == sd.src_off) dun1 += srcd;
            *reinterpret_cast<float2*>(&sDU[j][i]) = make_float2(dun0, dun1);
            *reinterpret_cast<float2*>(&sDQ[j][i]) = make_float2(dc.x + dun0, dc.y + dun1);
            if (own) *reinterpret_cast<float2*>(du2 + o) = make_float2(dun0, dun1);
        }
    }
    __syncthreads();
    // receivers of this tile: record row t = p_{t+2} (core/seis_forward2.py:249)
    const int tile = by * tiles_x + bx;
    const int r0 = a.tile_rec_start[tile], r1 = a.tile_rec_start[tile + 1];
    for (int k = r0 + tid; k < r1; k += kThreads) {
        const int rr = a.tile_rec_list[k];
        const int off = a.rec_off[rr];
        const long long ro = ((long long)slot * g.nt + t) * g.nrec + rr;
        a.rec[ro] = sQ[off / g.pitch - z0 + 2][off % g.pitch - x0 + 2];
        if (TAN) a.drec[ro] = sDQ[off / g.pitch - z0 + 2][off % g.pitch - x0 + 2];
    }

    // step t+1 on the tile
    const int xx = 2 * threadIdx.x;
    const int x = x0 + xx;
    if (x < g.NX) {
#pragma unroll
        for (int r = 0; r < kRPTile; ++r) {
            const int zz = threadIdx.y + r * kBZ;
            const int z = z0 + zz;
            if (z >= g.NZ) continue;
            const int i = z * g.pitch + x;
            float2 c;
            const float2 L = lap_pair(sQ, zz + 2, xx + 2, c);
            const float2 aa = __ldg(reinterpret_cast<const float2*>(al + i));
            const float om0 = one_minus_kappa(kf, z, x, a.dampx, a.dampz, g);
            const float om1 = one_minus_kappa(kf, z, x + 1, a.dampx, a.dampz, g);
            const float2 ucp = *reinterpret_cast<const float2*>(&sU[zz + 2][xx + 2]);
            const float uc0 = ucp.x, uc1 = ucp.y;
            const float2 un = fwd_increment(make_float2(om0, om1), ucp, aa, L);
            float un0 = un.x, un1 = un.y;
            if (i == sd.src_off) un0 += src2;
            if (i + 1 == sd.src_off) un1 += src2;
            const float2 un2 = make_float2(un0, un1);
            *reinterpret_cast<float2*>(u3 + i) = un2;
            *reinterpret_cast<float2*>(p3 + i) = add2(c, un2);
            if (TAN) {
                float2 dc;
                const float2 dL = lap_pair(sDQ, zz + 2, xx + 2, dc);
                const float2 ad = __ldg(reinterpret_cast<const float2*>(ald + i));
                const float kd0 = __fmul_rn(kdf, damp_at(z, x, a.dampx, a.dampz, g));
                const float kd1 = __fmul_rn(kdf, damp_at(z, x + 1, a.dampx, a.dampz, g));
                float dun0 = tan_increment(om0, sDU[zz + 2][xx + 2], aa.x, dL.x, ad.x, L.x, kd0, uc0);
                float dun1 = tan_increment(om1, sDU[zz + 2][xx + 3], aa.y, dL.y, ad.y, L.y, kd1, uc1);
                if (i == sd.src_off) dun0 += srcd2;
                if (i + 1 == sd.src_off) dun1 += srcd2;
                *reinterpret_cast<float2*>(du3 + i) = make_float2(dun0, dun1);
                *reinterpret_cast<float2*>(dp3 + i) = make_float2(dc.x + dun0, dc.y + dun1);
            }
        }
    }
    // record row t+1 = p_{t+3}, from this block's own writes
    if (r1 > r0) {
        __syncthreads();
        for (int k = r0 + tid; k < r1; k += kThreads) {
            const int rr = a.tile_rec_list[k];
            const long long ro = ((long long)slot * g.nt + t + 1) * g.nrec + rr;
            a.rec[ro] = p3[a.rec_off[rr]];
            if (TAN) a.drec[ro] = dp3[a.rec_off[rr]];
        }
    }
}

template <bool TAN>
__global__ void __launch_bounds__(kThreads, TAN ? 3 : 6) fwd_step2_kernel(FwdArgs a, int t)
{
    extern __shared__ __align__(16) float fsm[];
    fwd_step2_tile<TAN>(a, t, blockIdx.z, blockIdx.x, blockIdx.y, gridDim.x, fsm);
}

template <int HOIST = kRPTile>
__device__ __forceinline__ void adj_step2_tile(const AdjArgs& a, int t, int slot, int bx, int by, int tiles_x,
                                               float* fsm)
{
    float (*sAL)[kFW] = reinterpret_cast<float (*)[kFW]>(fsm);             // alpha, then alpha lambda_{t+3},
                                                                            // halo 4; then the seeds of row t-1
    float (*sLam)[kFW] = sAL + kFH;                                         // lambda_{t+3}, halo 4
    float (*sL)[kFW] = reinterpret_cast<float (*)[kFW]>(&sLam[2][2]);       // its halo-2 window: lambda_{t+3}
                                                                            // -> lambda_{t+2} in place
    float (*sB)[kSW] = reinterpret_cast<float (*)[kSW]>(fsm + 2 * kFH * kFW);   // alpha lambda_{t+2}
    float (*sM)[kSW] = sB + kSH;                                            // seeds of row t -> mu_{t+2}
    const ShotDesc sd = a.shots[slot];
    if (!sd.active) return;
    const GridDev& g = a.g;
    const int x0 = bx * kTX, z0 = by * kTZ;
    const long long NP = g.NP;
    const int tid = threadIdx.y * kBX + threadIdx.x;
    const float* lam3 = a.lam + (long long)slot * 3 * NP + (long long)(t % 3) * NP;          // lambda_{t+3}
    const float* mu3 = a.mu + (long long)slot * 3 * NP + (long long)(t % 3) * NP;            // mu_{t+3}
    float* lam1 = a.lam + (long long)slot * 3 * NP + (long long)((t + 1) % 3) * NP;          // lambda_{t+1}
    float* mu1 = a.mu + (long long)slot * 3 * NP + (long long)((t + 1) % 3) * NP;            // mu_{t+1}
    const float* al = a.alpha + (long long)sd.model * NP;
    const float kf = __ldg(a.kfac + sd.model);

    // this thread's step-t pairs: their mu_{t+3} and alpha loads issued up front
    float2 m3[kFusedTasks], av[kFusedTasks];
#pragma unroll
    for (int it = 0; it < kFusedTasks; ++it) {
        const int k = tid + it * kThreads;
        m3[it] = av[it] = make_float2(0.0f, 0.0f);
        if (k < kSH * (kSW / 2)) {
            const int j = k / (kSW / 2), i = 2 * (k - j * (kSW / 2));
            const long long o = (long long)wrap_once(z0 - 2 + j, g.NZ) * g.pitch + wrap_once(x0 - 2 + i, g.NX);
            m3[it] = *reinterpret_cast<const float2*>(mu3 + o);
            av[it] = __ldg(reinterpret_cast<const float2*>(al + o));
        }
    }
    // stage: lambda_{t+3} and alpha (halo 4), 8-byte asynchronous copies; seeds of row t
    for (int k = tid; k < kSH * kSW; k += kThreads) (&sM[0][0])[k] = 0.0f;
#pragma unroll
    for (int j = threadIdx.y; j < kFH; j += kBZ) {
        const long long rowo = (long long)wrap_once(z0 - 4 + j, g.NZ) * g.pitch;
#pragma unroll
        for (int q = threadIdx.x; q < kFW / 2; q += kBX) {
            const long long o = rowo + wrap_once(x0 - 4 + 2 * q, g.NX);
            async_copy8(&sLam[j][2 * q], lam3 + o);
            async_copy8(&sAL[j][2 * q], al + o);
        }
    }
    async_copies_wait();
    __syncthreads();
    // alpha lambda_{t+3} in place of alpha
    for (int k = tid; k < kFH * kFW / 2; k += kThreads) {
        float2* av2 = reinterpret_cast<float2*>(&sAL[0][0]) + k;
        const float2 lv = reinterpret_cast<const float2*>(&sLam[0][0])[k];
        const float2 aa = *av2;
        *av2 = make_float2(__fmul_rn(aa.x, lv.x), __fmul_rn(aa.y, lv.y));
    }
    __syncthreads();
    // seeds of row t on the tile + halo 2 (receivers there, periodic); they enter a
    // point's update exactly as in adj_step_kernel: added when the point's own tile
    // holds receivers
    for (int k = tid; k < g.nrec; k += kThreads) {
        const int off = a.rec_off[k];
        const int rz = wrap_once(off / g.pitch - (z0 - 2), g.NZ), rx = wrap_once(off % g.pitch - (x0 - 2), g.NX);
        if (rz < kSH && rx < kSW) sM[rz][rx] = a.seed[((long long)slot * g.nt + t) * g.nrec + k];
    }
    __syncthreads();
    const int tile = by * tiles_x + bx;
    const bool has_rec = a.tile_rec_start[tile + 1] > a.tile_rec_start[tile];

    // step t on the tile + halo 2
#pragma unroll
    for (int it = 0; it < kFusedTasks; ++it) {
        const int k = tid + it * kThreads;
        if (k >= kSH * (kSW / 2)) break;
        const int j = k / (kSW / 2), i = 2 * (k - j * (kSW / 2));
        const int z = wrap_once(z0 - 2 + j, g.NZ), x = wrap_once(x0 - 2 + i, g.NX);
        float2 cdummy;
        const float2 Lm = lap_pair<kFW>(sAL, j + 2, i + 2, cdummy);
        const float om0 = one_minus_kappa(kf, z, x, a.dampx, a.dampz, g);
        const float om1 = one_minus_kappa(kf, z, x + 1, a.dampx, a.dampz, g);
        const float2 mm = fma2(make_float2(om0, om1), m3[it], Lm);
        float m_0 = mm.x, m_1 = mm.y;
        const int tt = (z / kTZ) * tiles_x + x / kTX;       // the point's own tile
        if (a.tile_rec_start[tt + 1] > a.tile_rec_start[tt]) {
            m_0 += sM[j][i];
            m_1 += sM[j][i + 1];
        }
        const float2 ll = add2(*reinterpret_cast<const float2*>(&sL[j][i]), make_float2(m_0, m_1));
        *reinterpret_cast<float2*>(&sL[j][i]) = ll;
        *reinterpret_cast<float2*>(&sM[j][i]) = make_float2(m_0, m_1);
        *reinterpret_cast<float2*>(&sB[j][i]) = mul2(av[it], ll);
    }
    __syncthreads();
    // seeds of row t-1 on the tile, in the (now free) staging area
    float (*sS)[kTX] = reinterpret_cast<float (*)[kTX]>(fsm);
    if (has_rec) {
        for (int k = tid; k < kTZ * kTX; k += kThreads) (&sS[0][0])[k] = 0.0f;
        __syncthreads();
        for (int k = a.tile_rec_start[tile] + tid; k < a.tile_rec_start[tile + 1]; k += kThreads) {
            const int rr = a.tile_rec_list[k];
            const int off = a.rec_off[rr];
            sS[off / g.pitch - z0][off % g.pitch - x0] = a.seed[((long long)slot * g.nt + t - 1) * g.nrec + rr];
        }
        __syncthreads();
    }

    // step t-1 on the tile, and both steps' gradient terms
    const float* u2 = a.u + (long long)slot * a.u_slot_stride + (long long)((t + 1) % a.ulevels) * NP;  // u_{t+2}
    const float* u1 = a.u + (long long)slot * a.u_slot_stride + (long long)(t % a.ulevels) * NP;        // u_{t+1}
    const float* u0 = a.u + (long long)slot * a.u_slot_stride + (long long)((t - 1) % a.ulevels) * NP;  // u_t
    float* gv = a.gv + (long long)slot * NP;
    float* gk = a.gk + (long long)slot * NP;
    const int xx = 2 * threadIdx.x;
    const int x = x0 + xx;
    if (x >= g.NX) return;       // NX even: both columns of the pair are inside
    // the history and gradient-sum loads of HOIST rows at a time, issued before any of
    // their stores (which the compiler must assume could alias them): one global latency
    // per HOIST rows instead of one per row
    static_assert(kRPTile % HOIST == 0, "rows per thread in whole batches");
    float2 A2[kRPTile], A1[kRPTile], A0[kRPTile], GV[kRPTile], GK[kRPTile];
#pragma unroll
    for (int r = 0; r < kRPTile; ++r) {
        if (HOIST > 1 && r % HOIST == 0) {
#pragma unroll
            for (int h = r; h < r + HOIST; ++h) {
                const int z = z0 + threadIdx.y + h * kBZ;
                if (z >= g.NZ) continue;
                const int i = z * g.pitch + x;
                A2[h] = *reinterpret_cast<const float2*>(u2 + i);
                A1[h] = *reinterpret_cast<const float2*>(u1 + i);
                A0[h] = *reinterpret_cast<const float2*>(u0 + i);
                GV[h] = *reinterpret_cast<const float2*>(gv + i);
                GK[h] = *reinterpret_cast<const float2*>(gk + i);
            }
        }
        const int zz = threadIdx.y + r * kBZ;
        const int z = z0 + zz;
        if (z >= g.NZ) continue;
        const int i = z * g.pitch + x;
        float2 cdummy;
        const float2 Lm = lap_pair(sB, zz + 2, xx + 2, cdummy);
        const float om0 = one_minus_kappa(kf, z, x, a.dampx, a.dampz, g);
        const float om1 = one_minus_kappa(kf, z, x + 1, a.dampx, a.dampz, g);
        const float2 l2 = *reinterpret_cast<const float2*>(&sL[zz + 2][xx + 2]);          // lambda_{t+2}
        const float2 om = make_float2(om0, om1), nom = make_float2(-om0, -om1);
        const float2 mm = fma2(om, *reinterpret_cast<const float2*>(&sM[zz + 2][xx + 2]), Lm);
        float m_0 = mm.x, m_1 = mm.y;
        if (has_rec) {
            m_0 += sS[zz][xx];
            m_1 += sS[zz][xx + 1];
        }
        const float2 l1 = add2(l2, make_float2(m_0, m_1));                                   // lambda_{t+1}
        if (HOIST == 1) {
            A2[r] = *reinterpret_cast<const float2*>(u2 + i);
            A1[r] = *reinterpret_cast<const float2*>(u1 + i);
            A0[r] = *reinterpret_cast<const float2*>(u0 + i);
            GV[r] = *reinterpret_cast<const float2*>(gv + i);
            GK[r] = *reinterpret_cast<const float2*>(gk + i);
        }
        const float2 a2 = A2[r], a1 = A1[r], a0 = A0[r];
        float2 gvv = GV[r], gkk = GK[r];
        // step t, then step t-1 (the order of two single steps)
        gvv = fma2(l2, fma2(nom, a1, a2), gvv);
        gkk = fma2(l2, a1, gkk);
        gvv = fma2(l1, fma2(nom, a0, a1), gvv);
        gkk = fma2(l1, a0, gkk);
        *reinterpret_cast<float2*>(mu1 + i) = make_float2(m_0, m_1);
        *reinterpret_cast<float2*>(lam1 + i) = l1;
        *reinterpret_cast<float2*>(gv + i) = gvv;
        *reinterpret_cast<float2*>(gk + i) = gkk;
    }
}

template <int HOIST>
__global__ void __launch_bounds__(kThreads) adj_step2_kernel(AdjArgs a, int t)
{
    extern __shared__ __align__(16) float fsm[];
    adj_step2_tile<HOIST>(a, t, blockIdx.z, blockIdx.x, blockIdx.y, gridDim.x, fsm);
}

// Checkpoint save / restore: for every active slot copy n floats from
// src + slot*src_stride to dst + slot*dst_stride (offsets folded into the pointers).
__global__ void slot_copy_kernel(const ShotDesc* __restrict__ shots, long long n, const float* __restrict__ src,
                                 long long src_stride, float* __restrict__ dst, long long dst_stride)
{
    const int slot = blockIdx.y;
    if (!shots[slot].active) return;
    const float* s = src + (long long)slot * src_stride;
    float* d = dst + (long long)slot * dst_stride;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        d[i] = s[i];
}

}  // namespace
}  // namespace seis
