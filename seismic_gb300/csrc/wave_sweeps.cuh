// wave_sweeps.cuh -- persistent wavefront sweeps of the tiled path: one launch per sweep,
// over any number of shot groups of any geometries (the uneven batch in one launch).
//
// A sweep is a program of stages per shot slot -- two forward steps (fwd_step2_tile), one
// forward step, two or one reverse steps (adj_step2_tile / adj_step_tile), or a checkpoint
// copy -- each stage over every tile of the slot's grid.  The launch's work items are the
// (stage, slot, tile) triples of all groups, dequeued by the resident blocks from one
// atomic counter in group-major, stage-major order.  An item runs when the 3 x 3 tiles
// around it (periodic; 5 x 5 where a last tile is narrower than the 4-cell halo) have
// finished the slot's previous stage; every stage reads the previous stages' fields
// only there and writes only its own tile, and the three-level rotations are never
// overwritten before the stage after their readers has run, so each item computes what
// the same stage of the per-step launches computes: the results are bitwise those of the
// graph of step launches (core/seis_forward2.py:211-314 per shot).
//
// Deadlock freedom: an item waits only for items dequeued before it, which are held by
// running blocks that do not wait for later items.  Every wait is bounded by the global
// timer; on a timeout the block raises the launch's abort flag and bit 8 of the error word
// of every engine in the launch, and every block stops at its next dequeue or wait (the
// launch's results are invalid).
//
// Stage-major order within a group keeps the group's fields in L2 while its stages
// advance (the host sizes groups to a few slots of a large grid); groups follow one
// another in the queue without a barrier.
#pragma once
#include "sweep_kernels.cuh"

namespace seis {
namespace {

enum : int { kWaveF2 = 0, kWaveF1 = 1, kWaveA2 = 2, kWaveA1 = 3, kWaveCopy = 4 };

struct WaveStage {
    int kind;       // kWave*
    int t;          // time step of the stage (its first step for two-step stages)
    int copy;       // kWaveCopy: index into the group's copy table
    int pad;
};

// Checkpoint copy of one field level: slot s copies src + s*src_stride to dst + s*dst_stride.
struct WaveCopy {
    const float* src;
    float* dst;
    long long src_stride, dst_stride;
};

struct WaveGroup {
    const WaveStage* prog;  // [nstages]
    const WaveCopy* copies;
    int* progress;          // [nslots][tiles]: stages completed (zeroed before the launch)
    int* err;               // the group's engine's sticky error word
    long long first;        // the group's first item in the launch's queue
    int nstages, slot0, nslots, tiles_x, tiles_z;
    int reach;              // tiles a stage's 4-cell halo reaches: 1, or 2 next to a last tile
                            // narrower than 4 cells
    int args;               // index of the group's engine's arguments in the launch's parameters
    int pad0;               // explicit: group tables are cached by their bytes
};
static_assert(sizeof(WaveGroup) == 72 && sizeof(WaveStage) == 16 && sizeof(WaveCopy) == 32,
              "wavefront tables without implicit padding");

struct WaveLaunch {
    const WaveGroup* groups;   // sorted by first
    int ngroups;
    long long total;           // items of all groups
    unsigned long long* next;  // dequeue counter (zeroed before the launch)
    int* abort;                // raised by a timed-out wait (zeroed before the launch)
};

// Kernel parameters of a launch: the engines' sweep arguments live in the constant bank,
// like the step kernels' (a shared-memory copy costs registers and spills).  Launches
// over more engines are split.
constexpr int kMaxWaveArgs = 64;
template <int MODE>
struct WaveParams {
    WaveLaunch L;
    FwdArgs f[kMaxWaveArgs];
    AdjArgs a[MODE == 2 ? kMaxWaveArgs : 1];
};

constexpr unsigned long long kWaveTimeoutNs = 2000000000ull;
constexpr int kWaveErrBit = 8;

// Progress counters: published with release semantics after the block's barrier (so
// every thread's writes of the item precede them), polled with acquire semantics before
// the block's barrier (so every thread's later loads see the neighbours' fields).
__device__ __forceinline__ int ld_acquire(const int* p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(int* p, int v)
{
    asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long wave_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Bounded wait until *flag >= need; false on a timeout or once another block aborted.
__device__ __forceinline__ bool wave_wait(const int* flag, int need, const int* abort)
{
    if (ld_acquire(flag) >= need) return true;
    const unsigned long long t0 = wave_ns();
    for (unsigned i = 1;; ++i) {
        __nanosleep(32);
        if (ld_acquire(flag) >= need) return true;
        if ((i & 31u) == 0) {
            if (*(volatile const int*)abort) return false;
            if (wave_ns() - t0 > kWaveTimeoutNs) return false;
        }
    }
}

// Checkpoint copy of tile (bx, by) of one slot (grid points only; the pitch's padding
// columns are never read).
__device__ __forceinline__ void wave_copy_tile(const WaveCopy& c, const GridDev& g, int slot, int bx, int by)
{
    const float* s = c.src + (long long)slot * c.src_stride;
    float* d = c.dst + (long long)slot * c.dst_stride;
    const int tid = threadIdx.y * kBX + threadIdx.x;
    for (int k = tid; k < kTZ * (kTX / 2); k += kThreads) {
        const int j = k / (kTX / 2), x = bx * kTX + 2 * (k - j * (kTX / 2)), z = by * kTZ + j;
        if (z >= g.NZ || x >= g.NX) continue;
        const long long o = (long long)z * g.pitch + x;
        if (x + 1 < g.NX) *reinterpret_cast<float2*>(d + o) = *reinterpret_cast<const float2*>(s + o);
        else d[o] = s[o];
    }
}

// MODE 0: forward sweep, 1: forward + tangent, 2: adjoint sweep (with the checkpointed
// adjoint's recomputed forward segments).  Dynamic shared memory: wave_smem<MODE>().
template <int MODE>
constexpr int wave_smem()
{
    return MODE == 1 ? fused_fwd_smem<true>()
                     : (MODE == 0 ? fused_fwd_smem<false>()
                                  : (kFusedAdjSmem > fused_fwd_smem<false>() ? kFusedAdjSmem : fused_fwd_smem<false>()));
}

// MINB: resident blocks per SM the registers are sized for (the step kernels: 6 forward,
// 3 forward + tangent, 4 reverse).
//
// Thread 0 schedules: it takes the next item from the counter while the block still works
// on the current one, and decodes it (group, stage, slot, tile) into shared memory.
template <int MODE, int MINB>
__global__ void __launch_bounds__(kThreads, MINB) wave_sweep_kernel(const __grid_constant__ WaveParams<MODE> P)
{
    extern __shared__ __align__(16) float wsm[];
    __shared__ struct {
        int* done;                  // progress counters of the item's slot
        const WaveCopy* copies;
        int q, slot, tile, bx, by, tiles_x, tiles_z, reach, args, group, stop;
        WaveStage st;
        long long nxt, gfirst, gend;   // thread 0's scheduling state (kept out of registers)
    } s;
    const WaveLaunch& L = P.L;
    constexpr bool TAN = MODE == 1;
    const int tid = threadIdx.y * kBX + threadIdx.x;
    if (tid == 0) {
        s.nxt = (long long)atomicAdd(L.next, 1ull);
        s.gfirst = s.gend = 0;
        s.group = -1;
    }
    for (;;) {
        if (tid == 0) {
            const long long item = s.nxt;
            s.stop = item >= L.total || *(volatile const int*)L.abort;
            if (!s.stop) {
                s.nxt = (long long)atomicAdd(L.next, 1ull);     // the next item, in flight during this one
                if (item < s.gfirst || item >= s.gend) {
                    int lo = 0, hi = L.ngroups - 1;
                    while (lo < hi) {
                        const int mid = (lo + hi + 1) >> 1;
                        if (L.groups[mid].first <= item) lo = mid;
                        else hi = mid - 1;
                    }
                    const WaveGroup& G = L.groups[lo];
                    s.gfirst = G.first;
                    s.gend = G.first + (long long)G.nstages * G.nslots * G.tiles_x * G.tiles_z;
                    s.group = lo;
                }
                const WaveGroup& G = L.groups[s.group];
                const int tx = G.tiles_x, tz = G.tiles_z, tiles = tx * tz;
                const long long per_stage = (long long)G.nslots * tiles;
                const long long local = item - s.gfirst;
                const int q = (int)(local / per_stage);
                const int rem = (int)(local - (long long)q * per_stage);
                const int ls = rem / tiles, tile = rem - ls * tiles;
                s.done = G.progress + (long long)ls * tiles;
                s.copies = G.copies;
                s.q = q;
                s.slot = G.slot0 + ls;
                s.tile = tile;
                s.bx = tile % tx;
                s.by = tile / tx;
                s.tiles_x = tx;
                s.tiles_z = tz;
                s.reach = G.reach;
                s.args = G.args;
                s.st = G.prog[q];
            }
        }
        __syncthreads();
        if (s.stop) break;
        // the tiles within `reach` of this one (5 x 5, or 3 x 3 where no last tile is
        // narrower than the 4-cell halo) have finished stage q-1
        const int q = s.q, bx = s.bx, by = s.by, tx = s.tiles_x, tz = s.tiles_z;
        bool ok = true;
        const int w = 2 * s.reach + 1;
        if (q > 0 && tid < w * w) {
            const int nx = (bx + tid % w - s.reach + 2 * tx) % tx;
            const int nz = (by + tid / w - s.reach + 2 * tz) % tz;
            ok = wave_wait(s.done + nz * tx + nx, q, L.abort);
        }
        if (!ok && atomicExch(L.abort, 1) == 0)
            for (int k = 0; k < L.ngroups; ++k) atomicOr(L.groups[k].err, kWaveErrBit);   // every engine of the launch
        if (__syncthreads_or(!ok)) break;
        const WaveStage st = s.st;
        const int slot = s.slot, ai = s.args;
        if (st.kind == kWaveF2) {
            fwd_step2_tile<TAN>(P.f[ai], st.t, slot, bx, by, tx, wsm);
        } else if (st.kind == kWaveF1) {
            float (*sp)[kSW] = reinterpret_cast<float (*)[kSW]>(wsm);
            fwd_step_tile<TAN>(P.f[ai], st.t, slot, bx, by, tx, sp, sp + kSH);
        } else if (MODE == 2 && st.kind == kWaveA2) {
            adj_step2_tile<1>(P.a[ai], st.t, slot, bx, by, tx, wsm);   // at 64 registers a deeper hoist spills
        } else if (MODE == 2 && st.kind == kWaveA1) {
            float (*sm)[kSW] = reinterpret_cast<float (*)[kSW]>(wsm);
            adj_step_tile(P.a[ai], st.t, slot, bx, by, tx, sm, reinterpret_cast<float (*)[kTX]>(wsm + kSH * kSW));
        } else if (st.kind == kWaveCopy) {
            if (P.f[ai].shots[slot].active) wave_copy_tile(s.copies[st.copy], P.f[ai].g, slot, bx, by);
        }
        __syncthreads();
        if (tid == 0) {
            __threadfence();
            st_release(s.done + s.tile, q + 1);
        }
    }
}

}  // namespace
}  // namespace seis
