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

constexpr int kTX = 32;           // tile columns (one warp wide)
constexpr int kTZ = 16;           // tile rows
constexpr int kBZ = 8;            // block rows; each thread owns kTZ/kBZ points
constexpr int kThreads = kTX * kBZ;
constexpr int kSW = kTX + 4;      // staged tile width with the 2-cell halo
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
    float* p;                // [slot][2][NP]
    float* u;                // [slot][ulevels][NP]
    long long u_slot_stride;
    int ulevels;             // 2 (ring) or nt+1 (history kept for the adjoint)
    float* dp;               // [slot][2][NP]  (tangent)
    float* du;               // [slot][2][NP]  (tangent)
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
    float* lam;              // [slot][2][NP]
    float* mu;               // [slot][NP]
    float* gv;               // [slot][NP]
    float* gk;               // [slot][NP]
    const float* seed;       // [slot][nt][nrec]
    const int* tile_rec_start;
    const int* tile_rec_list;
    const int* rec_off;
};

__device__ __forceinline__ void stage_tile(float (*s)[kSW], const float* __restrict__ f, int z0, int x0,
                                           const GridDev& g)
{
    const int tid = threadIdx.y * kTX + threadIdx.x;
    for (int k = tid; k < kSH * kSW; k += kThreads) {
        const int j = k / kSW, i = k - j * kSW;
        const int gz = wrap_idx(z0 - 2 + j, g.NZ);
        const int gx = wrap_idx(x0 - 2 + i, g.NX);
        s[j][i] = f[(long long)gz * g.pitch + gx];
    }
}

// Full 4th-order Laplacian at tile-local centre (zz, xx) (halo offset included).
__device__ __forceinline__ float lap_tile(const float (*s)[kSW], int zz, int xx)
{
    const float c = s[zz][xx];
    const float t1 = (s[zz][xx + 1] + s[zz][xx - 1]) + (s[zz + 1][xx] + s[zz - 1][xx]);
    const float t2 = (s[zz][xx + 2] + s[zz][xx - 2]) + (s[zz + 2][xx] + s[zz - 2][xx]);
    return kC2 * (t1 - 4.0f * c) + kC3 * (t2 - 4.0f * c);
}

template <bool TAN>
__global__ void __launch_bounds__(kThreads) fwd_step_kernel(FwdArgs a, int t)
{
    __shared__ float sp[kSH][kSW];
    __shared__ float sdp[TAN ? kSH : 1][kSW];
    const int slot = blockIdx.z;
    const ShotDesc sd = a.shots[slot];
    if (!sd.active) return;
    const GridDev& g = a.g;
    const int x0 = blockIdx.x * kTX, z0 = blockIdx.y * kTZ;
    const long long NP = g.NP;

    const float* pcur = a.p + (long long)slot * 2 * NP + ((t + 1) & 1) * NP;
    float* pnext = a.p + (long long)slot * 2 * NP + (t & 1) * NP;
    const float* ucur = a.u + (long long)slot * a.u_slot_stride + (long long)(t % a.ulevels) * NP;
    float* unext = a.u + (long long)slot * a.u_slot_stride + (long long)((t + 1) % a.ulevels) * NP;
    const float* dpcur = nullptr;
    float* dpnext = nullptr;
    const float* ducur = nullptr;
    float* dunext = nullptr;
    if (TAN) {
        dpcur = a.dp + (long long)slot * 2 * NP + ((t + 1) & 1) * NP;
        dpnext = a.dp + (long long)slot * 2 * NP + (t & 1) * NP;
        ducur = a.du + (long long)slot * 2 * NP + (t & 1) * NP;
        dunext = a.du + (long long)slot * 2 * NP + ((t + 1) & 1) * NP;
    }
    stage_tile(sp, pcur, z0, x0, g);
    if (TAN) stage_tile(sdp, dpcur, z0, x0, g);
    __syncthreads();

    const float* al = a.alpha + (long long)sd.model * NP;
    const float kf = __ldg(a.kfac + sd.model);
    const float* ald = TAN ? a.alpha_d + (long long)sd.model * NP : nullptr;
    const float kdf = TAN ? __ldg(a.kdfac + sd.model) : 0.0f;
    const float src = __ldg(a.smod + (long long)slot * g.nt + t);
    const float src_d = TAN ? __ldg(a.smod_d + (long long)slot * g.nt + t) : 0.0f;
    const int x = x0 + threadIdx.x;
#pragma unroll
    for (int r = 0; r < kTZ / kBZ; ++r) {
        const int zz = threadIdx.y + r * kBZ;
        const int z = z0 + zz;
        if (x < g.NX && z < g.NZ) {
            const long long i = (long long)z * g.pitch + x;
            const float L = lap_tile(sp, zz + 2, threadIdx.x + 2);
            const float kap = kf * damp_at(z, x, a.dampx, a.dampz, g);
            const float om = 1.0f - kap;
            const float aa = __ldg(al + i);
            const float uc = ucur[i];
            float un = om * uc + aa * L;
            const bool at_src = (i == sd.src_off);
            if (at_src) un += src;
            unext[i] = un;
            pnext[i] = sp[zz + 2][threadIdx.x + 2] + un;
            if (TAN) {
                const float dL = lap_tile(sdp, zz + 2, threadIdx.x + 2);
                const float kd = kdf * damp_at(z, x, a.dampx, a.dampz, g);
                float dun = om * ducur[i] + aa * dL + __ldg(ald + i) * L - kd * uc;
                if (at_src) dun += src_d;
                dunext[i] = dun;
                dpnext[i] = sdp[zz + 2][threadIdx.x + 2] + dun;
            }
        }
    }
    // receiver gather of this tile (record row t = level t+2, core/seis_forward2.py:249)
    const int tile = blockIdx.y * gridDim.x + blockIdx.x;
    const int r0 = a.tile_rec_start[tile], r1 = a.tile_rec_start[tile + 1];
    if (r1 > r0) {
        __syncthreads();
        const int tid = threadIdx.y * kTX + threadIdx.x;
        for (int k = r0 + tid; k < r1; k += kThreads) {
            const int rr = a.tile_rec_list[k];
            const long long o = ((long long)slot * g.nt + t) * g.nrec + rr;
            a.rec[o] = pnext[a.rec_off[rr]];
            if (TAN) a.drec[o] = dpnext[a.rec_off[rr]];
        }
    }
}

// Reverse step t (t = nt-1 .. 0): lambda_{t+2} from lambda_{t+3}, mu_{t+3}.
__global__ void __launch_bounds__(kThreads) adj_step_kernel(AdjArgs a, int t)
{
    __shared__ float sm[kSH][kSW];
    __shared__ float sseed[kTZ][kTX];
    const int slot = blockIdx.z;
    const ShotDesc sd = a.shots[slot];
    if (!sd.active) return;
    const GridDev& g = a.g;
    const int x0 = blockIdx.x * kTX, z0 = blockIdx.y * kTZ;
    const long long NP = g.NP;
    const float* lprev = a.lam + (long long)slot * 2 * NP + ((t + 1) & 1) * NP;  // lambda_{t+3}
    float* lnext = a.lam + (long long)slot * 2 * NP + (t & 1) * NP;             // lambda_{t+2}
    const float* al = a.alpha + (long long)sd.model * NP;
    const int tid = threadIdx.y * kTX + threadIdx.x;

    for (int k = tid; k < kSH * kSW; k += kThreads) {
        const int j = k / kSW, i = k - j * kSW;
        const long long o = (long long)wrap_idx(z0 - 2 + j, g.NZ) * g.pitch + wrap_idx(x0 - 2 + i, g.NX);
        sm[j][i] = __ldg(al + o) * lprev[o];
    }
    for (int k = tid; k < kTZ * kTX; k += kThreads) (&sseed[0][0])[k] = 0.0f;
    const int tile = blockIdx.y * gridDim.x + blockIdx.x;
    const int r0 = a.tile_rec_start[tile], r1 = a.tile_rec_start[tile + 1];
    if (r1 > r0) {
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
    float* mu = a.mu + (long long)slot * NP;
    float* gv = a.gv + (long long)slot * NP;
    float* gk = a.gk + (long long)slot * NP;
    const int x = x0 + threadIdx.x;
#pragma unroll
    for (int r = 0; r < kTZ / kBZ; ++r) {
        const int zz = threadIdx.y + r * kBZ;
        const int z = z0 + zz;
        if (x < g.NX && z < g.NZ) {
            const long long i = (long long)z * g.pitch + x;
            const float Lm = lap_tile(sm, zz + 2, threadIdx.x + 2);
            const float om = 1.0f - kf * damp_at(z, x, a.dampx, a.dampz, g);
            const float m = om * mu[i] + Lm + sseed[zz][threadIdx.x];
            const float lam = lprev[i] + m;
            mu[i] = m;
            lnext[i] = lam;
            const float a1 = u1[i];
            gv[i] += lam * (u2[i] - om * a1);
            gk[i] += lam * a1;
        }
    }
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
