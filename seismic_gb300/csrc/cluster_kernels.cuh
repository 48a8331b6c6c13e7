// cluster_kernels.cuh -- cluster-resident, time-fused sweeps (sm_103a).
//
// One thread-block cluster of C CTAs owns one shot at a time and keeps its
// padded wavefield in the CTAs' shared memory for the whole time loop: CTA k
// holds a band of R consecutive rows (the last band may be shorter), the
// time loop runs inside the kernel, and the only per-step traffic to HBM is
// the forward increment history (written by the forward sweep, read back by
// the adjoint sweep) and the receiver records / seeds.
//
// Per step each CTA
//   1. applies the stencil to its band from shared memory (rows -2..R+1 of the
//      current buffer; rows -2,-1 and R,R+1 are halo copies of the
//      neighbouring bands, periodic across the whole padded grid as in the
//      reference's wrap, core/seis_forward2.py:395-403),
//   2. writes its new rows into the next buffer and PUSHES its first two and
//      last two rows into the neighbours' halo rows of that buffer through
//      distributed shared memory (mapa + st.shared::cluster),
//   3. meets the rest of the cluster at one barrier.cluster (release/acquire),
//      which both publishes the pushes and retires all reads of the buffer
//      that the next step overwrites.
// Each thread owns one column x and a strip of RPT consecutive rows of its
// band; it walks the strip with a 5-row sliding window in registers (vertical
// neighbours), reads the horizontal neighbours from shared memory at
// compile-time offsets (the row pitch SP is a template parameter; two ghost
// columns on each side carry the periodic wrap in x), and keeps its per-point
// private state (the increments u, or the adjoint's lambda, mu and gradient
// sums) in registers.  Work that concerns few points -- halo pushes, ghost
// columns, the source, receiver gathers and seeds -- runs outside the point
// loop or in warp-uniform variants of it, so the common warps run a lean loop.
//
// The adjoint additionally streams the forward increments u_{t+1}, u_{t+2}
// of its band back from HBM with 1-D TMA bulk copies (cp.async.bulk +
// mbarrier complete_tx) into a 3-deep shared-memory ring, one step ahead of
// use.  Every mbarrier wait is bounded: on timeout the kernel records an error
// and keeps meeting the cluster barriers (so no CTA is left waiting), and the
// host reports the error.
#pragma once
#include <stdint.h>

#include "common.cuh"

namespace seis {
namespace {

// ---------------------------------------------------------------------------
// PTX helpers: cluster, distributed shared memory, mbarrier, TMA bulk copy
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned cl_rank()
{
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ unsigned cl_id()
{
    unsigned r;
    asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
    return r;
}
__device__ __forceinline__ unsigned cl_count()
{
    unsigned r;
    asm volatile("mov.u32 %0, %%nclusterid.x;" : "=r"(r));
    return r;
}
__device__ __forceinline__ void cl_sync()
{
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// Split form: arrive publishes this thread's earlier shared-memory writes
// (local and remote); work issued between arrive and wait (global stores,
// prefetches) overlaps the barrier and is not covered by the release.
__device__ __forceinline__ void cl_arrive()
{
    asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
}
__device__ __forceinline__ void cl_wait()
{
    asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ unsigned cl_map(unsigned local_addr, unsigned rank)
{
    unsigned r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(local_addr), "r"(rank));
    return r;
}
__device__ __forceinline__ void cl_store(unsigned cluster_addr, float v)
{
    asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(cluster_addr), "f"(v) : "memory");
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
// Non-blocking test of an mbarrier phase (test_wait never suspends the thread).
__device__ __forceinline__ bool mbar_test_wait(uint64_t* bar, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// 1-D bulk copy global -> this CTA's shared memory, completion counted on `bar`.
__device__ __forceinline__ void tma_load_1d(void* dst, const void* src, unsigned bytes, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

// Bounded wait on an mbarrier phase: false once kMbarTimeoutNs of wall time
// (the GPU's global timer) have passed without the phase completing.
constexpr unsigned long long kMbarTimeoutNs = 2000000000ull;
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity)
{
    if (mbar_test_wait(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    for (unsigned i = 1;; ++i) {
        if (mbar_test_wait(bar, parity)) return true;
        if ((i & 255u) == 0 && global_ns() - t0 > kMbarTimeoutNs) return false;
    }
}

// ---------------------------------------------------------------------------
// shared geometry of the cluster kernels
// ---------------------------------------------------------------------------
struct ClusterArgs {
    GridDev g;
    int R;                 // rows per band (the last band has NZ - (C-1) R)
    int G;                 // row groups (strips) per CTA; threads = G * SP
    int slots;             // shot slots of the chunk
    const ShotDesc* shots;
    const float* alpha;    // [model][NP]
    const float* kfac;     // [model]
    const float* dampx;    // [pitch]
    const float* dampz;    // [NZ]
    const int* rec_z;      // [nrec] padded rows
    const int* rec_x;      // [nrec] padded columns
    // forward
    const float* smod;     // [slot][nt]
    float* rec;            // [slot][nt][nrec]
    float* uhist;          // [slot][nt+1][NP] (forward writes levels 1..nt, adjoint reads)
    long long u_slot_stride;
    int write_hist;
    // adjoint
    const float* seed;     // [slot][nt][nrec]
    float* gv;             // [slot][NP]
    float* gk;             // [slot][NP]
    int* err;              // error word: 1 = an mbarrier wait timed out
};

__device__ __forceinline__ int band_rows(int k, int R, int NZ)
{
    const int r = NZ - k * R;
    return r < R ? r : R;
}

// Per-CTA constants of a band: wavefield buffers are [R+4][SP] with band row
// r at buffer row r+2 and column x at buffer column x+2.
template <int SP>
struct Band {
    int k, Rk, R_up, z0, NX;
    unsigned up_rank, dn_rank;
    __device__ __forceinline__ static int at(int r, int x) { return (r + 2) * SP + x + 2; }
};

// Copy band rows 0,1 / Rk-2,Rk-1 of this thread's strip into the neighbours'
// halo rows of buffer `nb` (DSMEM pushes), and this thread's columns 0,1 /
// NX-2,NX-1 into the ghost columns of its own rows.  Reads back the values
// this thread just wrote.
template <int SP>
__device__ __forceinline__ void push_edges(float* nb, unsigned nb_addr, const Band<SP>& b, int r_begin, int nrows,
                                           int x)
{
    const int r_end = r_begin + nrows;
    const int ghost = x < 2 ? b.NX + 2 + x : (x >= b.NX - 2 ? x - (b.NX - 2) : -1);
    if (ghost >= 0)
        for (int r = r_begin; r < r_end; ++r) nb[(r + 2) * SP + ghost] = nb[Band<SP>::at(r, x)];
    const int rows[4] = {0, 1, b.Rk - 2, b.Rk - 1};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int r = rows[q];
        if (r < r_begin || r >= r_end || (q >= 2 && r < 2)) continue;   // rows 0,1 are pushed once
        const float v = nb[Band<SP>::at(r, x)];
        if (q < 2) cl_store(cl_map(nb_addr + 4u * (unsigned)Band<SP>::at(b.R_up + r, x), b.up_rank), v);
        if (r >= b.Rk - 2) cl_store(cl_map(nb_addr + 4u * (unsigned)Band<SP>::at(r - b.Rk, x), b.dn_rank), v);
    }
}

// Strip of the forward step: u' = (1-k) u + a Lap(p) [+ src], p' = p + u'.
// FULL: the strip has RPT rows; SRC: the strip may hold the source.
template <int RPT, int SP, bool FULL, bool SRC>
__device__ __forceinline__ void fwd_strip(const float* __restrict__ cb, float* __restrict__ nb,
                                          const float* __restrict__ A, const float* __restrict__ OM, float (&u)[RPT],
                                          int r_begin, int nrows, int x, int jsrc, float src)
{
    const float* col = cb + r_begin * SP + x + 2;   // buffer row r_begin = band row r_begin-2
    float w0 = col[0], w1 = col[SP], w2 = col[2 * SP], w3 = col[3 * SP];
    const float* a = A + r_begin * SP + x;
    const float* om = OM + r_begin * SP + x;
    float* out = nb + (r_begin + 2) * SP + x + 2;
#pragma unroll
    for (int j = 0; j < RPT; ++j) {
        if (FULL || j < nrows) {
            const float w4 = col[(j + 4) * SP];
            const float* row = col + (j + 2) * SP;
            const float c = w2;
            const float t1 = (row[1] + row[-1]) + (w3 + w1);
            const float t2 = (row[2] + row[-2]) + (w4 + w0);
            const float L = kC2 * (t1 - 4.0f * c) + kC3 * (t2 - 4.0f * c);
            float un = om[j * SP] * u[j] + a[j * SP] * L;
            if (SRC && j == jsrc) un += src;
            u[j] = un;
            out[j * SP] = c + un;
            w0 = w1; w1 = w2; w2 = w3; w3 = w4;
        }
    }
}

// ---------------------------------------------------------------------------
// forward sweep
// smem: P[2][R+4][SP] | A[R][SP] | OM[R][SP] | S[nt] | receivers of the band (3 x nrec ints) | count
// ---------------------------------------------------------------------------
template <int C, int RPT, int SP>
__global__ void __launch_bounds__(1024, 1) fwd_cluster_kernel(ClusterArgs a)
{
    extern __shared__ __align__(16) float sm[];
    const GridDev& g = a.g;
    const int R = a.R;
    Band<SP> b;
    b.k = (int)cl_rank();
    b.Rk = band_rows(b.k, R, g.NZ);
    b.up_rank = (unsigned)((b.k + C - 1) % C);
    b.dn_rank = (unsigned)((b.k + 1) % C);
    b.R_up = band_rows((int)b.up_rank, R, g.NZ);
    b.z0 = b.k * R;
    b.NX = g.NX;
    const int bufsz = (R + 4) * SP;
    float* P0 = sm;
    float* P1 = sm + bufsz;
    float* A = sm + 2 * bufsz;
    float* OM = A + R * SP;
    float* SRC = OM + R * SP;
    int* RL = (int*)(SRC + g.nt);          // [3][nrec]: band row, column, receiver id
    int* nrl = RL + 3 * g.nrec;
    const int tid = threadIdx.x;
    const int x = tid % SP, gg = tid / SP;
    const int r_begin = gg * RPT;
    const int nrows = max(0, min(RPT, b.Rk - r_begin));
    const bool live = x < g.NX && nrows > 0;
    const unsigned addr0 = smem_addr(P0), addr1 = smem_addr(P1);

    for (int slot = (int)cl_id(); slot < a.slots; slot += (int)cl_count()) {
        const ShotDesc sd = a.shots[slot];
        if (!sd.active) break;  // uniform across the cluster
        const float* al = a.alpha + (long long)sd.model * g.NP;
        const float kf = __ldg(a.kfac + sd.model);
        if (tid == 0) *nrl = 0;
        for (int i = tid; i < 2 * bufsz; i += blockDim.x) sm[i] = 0.0f;
        for (int i = tid; i < b.Rk * SP; i += blockDim.x) {
            const int r = i / SP, xx = i - r * SP;
            const int z = b.z0 + r;
            A[i] = xx < g.NX ? __ldg(al + (long long)z * g.pitch + xx) : 0.0f;
            OM[i] = xx < g.NX ? 1.0f - kf * damp_at(z, xx, a.dampx, a.dampz, g) : 0.0f;
        }
        const float* smod = a.smod + (long long)slot * g.nt;
        for (int i = tid; i < g.nt; i += blockDim.x) SRC[i] = __ldg(smod + i);
        __syncthreads();
        for (int i = tid; i < g.nrec; i += blockDim.x) {
            const int rz = __ldg(a.rec_z + i) - b.z0;
            if (rz >= 0 && rz < b.Rk) {
                const int q = atomicAdd(nrl, 1);
                RL[q] = rz;
                RL[g.nrec + q] = __ldg(a.rec_x + i);
                RL[2 * g.nrec + q] = i;
            }
        }
        const int sz = sd.src_off / g.pitch - b.z0, sx = sd.src_off % g.pitch;
        const int jsrc = (live && sx == x && sz >= r_begin && sz < r_begin + nrows) ? sz - r_begin : -1;
        const bool warp_src = __any_sync(0xffffffffu, jsrc >= 0);
        const bool full = nrows == RPT;
        float* rec = a.rec + (long long)slot * g.nt * g.nrec;
        float* hist = a.write_hist ? a.uhist + (long long)slot * a.u_slot_stride + (long long)b.z0 * g.pitch + x
                                   : nullptr;
        float u[RPT];
#pragma unroll
        for (int j = 0; j < RPT; ++j) u[j] = 0.0f;
        __syncthreads();
        const int nr = *nrl;
        cl_sync();

        for (int t = 0; t < g.nt; ++t) {
            const float* cb = ((t + 1) & 1) ? P1 : P0;   // p_{t+1}
            float* nb = (t & 1) ? P1 : P0;               // p_{t+2}
            const unsigned nb_addr = (t & 1) ? addr1 : addr0;
            // record row t-1 = p_{t+1}, complete in this CTA's buffer
            if (t > 0)
                for (int i = tid; i < nr; i += blockDim.x)
                    rec[(long long)(t - 1) * g.nrec + RL[2 * g.nrec + i]] = cb[Band<SP>::at(RL[i], RL[g.nrec + i])];
            if (live) {
                const float src = SRC[t];
                if (warp_src) {
                    if (full) fwd_strip<RPT, SP, true, true>(cb, nb, A, OM, u, r_begin, nrows, x, jsrc, src);
                    else fwd_strip<RPT, SP, false, true>(cb, nb, A, OM, u, r_begin, nrows, x, jsrc, src);
                } else {
                    if (full) fwd_strip<RPT, SP, true, false>(cb, nb, A, OM, u, r_begin, nrows, x, -1, 0.0f);
                    else fwd_strip<RPT, SP, false, false>(cb, nb, A, OM, u, r_begin, nrows, x, -1, 0.0f);
                }
                push_edges<SP>(nb, nb_addr, b, r_begin, nrows, x);
            }
            cl_arrive();
            // history stores overlap the cluster barrier
            if (live && hist) {
                float* h = hist + (long long)(t + 1) * g.NP + (long long)r_begin * g.pitch;
#pragma unroll
                for (int j = 0; j < RPT; ++j)
                    if (j < nrows) h[j * SP] = u[j];
            }
            cl_wait();
        }
        // last record row: p_{nt+1}
        const float* fb = ((g.nt + 1) & 1) ? P1 : P0;
        for (int i = tid; i < nr; i += blockDim.x)
            rec[(long long)(g.nt - 1) * g.nrec + RL[2 * g.nrec + i]] = fb[Band<SP>::at(RL[i], RL[g.nrec + i])];
        cl_sync();   // every CTA done with its buffers before the next slot clears them
    }
}

// Strip of the adjoint step:
//   mu = (1-k) mu + Lap(a lambda') [+ seed],  lambda = lambda' + mu,
//   Gv += lambda (u_{t+2} - (1-k) u_{t+1}),  Gk += lambda u_{t+1},  M' = a lambda.
template <int RPT, int SP, bool FULL, bool SEED>
__device__ __forceinline__ void adj_strip(const float* __restrict__ cb, float* __restrict__ nb,
                                          const float* __restrict__ A, const float* __restrict__ OM,
                                          const float* __restrict__ U1, const float* __restrict__ U2,
                                          float (&lam)[RPT], float (&mu)[RPT], float (&gv)[RPT], float (&gk)[RPT],
                                          int r_begin, int nrows, int x, int j0, float s0, int j1, float s1)
{
    const float* col = cb + r_begin * SP + x + 2;
    float w0 = col[0], w1 = col[SP], w2 = col[2 * SP], w3 = col[3 * SP];
    const int o0 = r_begin * SP + x;
    float* out = nb + (r_begin + 2) * SP + x + 2;
#pragma unroll
    for (int j = 0; j < RPT; ++j) {
        if (FULL || j < nrows) {
            const float w4 = col[(j + 4) * SP];
            const float* row = col + (j + 2) * SP;
            const float c = w2;
            const float t1 = (row[1] + row[-1]) + (w3 + w1);
            const float t2 = (row[2] + row[-2]) + (w4 + w0);
            const float L = kC2 * (t1 - 4.0f * c) + kC3 * (t2 - 4.0f * c);
            const int o = o0 + j * SP;
            const float om = OM[o];
            float m = om * mu[j] + L;
            if (SEED) {
                if (j == j0) m += s0;
                if (j == j1) m += s1;
            }
            const float lv = lam[j] + m;
            mu[j] = m;
            lam[j] = lv;
            const float a1 = U1[o];
            gv[j] += lv * (U2[o] - om * a1);
            gk[j] += lv * a1;
            out[j * SP] = A[o] * lv;
            w0 = w1; w1 = w2; w2 = w3; w3 = w4;
        }
    }
}

// ---------------------------------------------------------------------------
// adjoint sweep (t = nt-1 .. 0)
// smem: M[2][R+4][SP] (a*lambda) | A[R][SP] | OM[R][SP] | U[3][R][SP] | mbar[3]
// ---------------------------------------------------------------------------
template <int C, int RPT, int SP>
__global__ void __launch_bounds__(1024, 1) adj_cluster_kernel(ClusterArgs a)
{
    extern __shared__ __align__(16) float sm[];
    const GridDev& g = a.g;
    const int R = a.R;
    Band<SP> b;
    b.k = (int)cl_rank();
    b.Rk = band_rows(b.k, R, g.NZ);
    b.up_rank = (unsigned)((b.k + C - 1) % C);
    b.dn_rank = (unsigned)((b.k + 1) % C);
    b.R_up = band_rows((int)b.up_rank, R, g.NZ);
    b.z0 = b.k * R;
    b.NX = g.NX;
    const int bufsz = (R + 4) * SP;
    const int band = R * SP;
    float* M0 = sm;
    float* M1 = sm + bufsz;
    float* A = sm + 2 * bufsz;
    float* OM = A + band;
    float* U = OM + band;                                  // 3 levels of the band
    uint64_t* bars = (uint64_t*)(U + 3 * band);            // band*4 is a multiple of 128 bytes
    const int tid = threadIdx.x;
    const int x = tid % SP, gg = tid / SP;
    const int r_begin = gg * RPT;
    const int nrows = max(0, min(RPT, b.Rk - r_begin));
    const bool live = x < g.NX && nrows > 0;
    const bool full = nrows == RPT;
    const unsigned band_bytes = (unsigned)(b.Rk * SP * 4);
    const unsigned addr0 = smem_addr(M0), addr1 = smem_addr(M1);
    unsigned phase = 0u;    // bit i: parity of the next phase to wait for on barrier i
    bool failed = false;

    if (tid == 0) {
        for (int i = 0; i < 3; ++i) mbar_init(bars + i, 1);
        fence_mbar_init();
    }
    __syncthreads();

    for (int slot = (int)cl_id(); slot < a.slots; slot += (int)cl_count()) {
        const ShotDesc sd = a.shots[slot];
        if (!sd.active) break;
        const float* al = a.alpha + (long long)sd.model * g.NP;
        const float kf = __ldg(a.kfac + sd.model);
        const float* hist = a.uhist + (long long)slot * a.u_slot_stride + (long long)b.z0 * g.pitch;
        // prefetch levels nt (u_{nt+1}) and nt-1 (u_nt) for the first reverse step
        if (tid == 0) {
            fence_proxy_async();
            for (int l = g.nt; l >= g.nt - 1 && l >= 0; --l) {
                const int q = l % 3;
                mbar_expect_tx(bars + q, band_bytes);
                tma_load_1d(U + q * band, hist + (long long)l * g.NP, band_bytes, bars + q);
            }
        }
        for (int i = tid; i < 2 * bufsz; i += blockDim.x) sm[i] = 0.0f;
        for (int i = tid; i < b.Rk * SP; i += blockDim.x) {
            const int r = i / SP, xx = i - r * SP;
            const int z = b.z0 + r;
            A[i] = xx < g.NX ? __ldg(al + (long long)z * g.pitch + xx) : 0.0f;
            OM[i] = xx < g.NX ? 1.0f - kf * damp_at(z, xx, a.dampx, a.dampz, g) : 0.0f;
        }
        // receivers in this thread's strip (at most two)
        int j0 = -1, r0 = -1, j1 = -1, r1 = -1;
        if (live)
            for (int i = 0; i < g.nrec; ++i) {
                const int rz = __ldg(a.rec_z + i) - b.z0 - r_begin;
                if (__ldg(a.rec_x + i) != x || rz < 0 || rz >= nrows) continue;
                if (j0 < 0) { j0 = rz; r0 = i; }
                else if (j1 < 0) { j1 = rz; r1 = i; }
            }
        const bool warp_seed = __any_sync(0xffffffffu, j0 >= 0);
        const float* seed = a.seed + (long long)slot * g.nt * g.nrec;
        float s0 = j0 >= 0 ? __ldg(seed + (long long)(g.nt - 1) * g.nrec + r0) : 0.0f;
        float s1 = j1 >= 0 ? __ldg(seed + (long long)(g.nt - 1) * g.nrec + r1) : 0.0f;
        float lam[RPT], mu[RPT], gv[RPT], gk[RPT];
#pragma unroll
        for (int j = 0; j < RPT; ++j) lam[j] = mu[j] = gv[j] = gk[j] = 0.0f;
        // level nt is read (as u_{t+2}) from the first step on: wait for it here;
        // every later level is waited for at the step that first reads it
        if (!mbar_wait_bounded(bars + g.nt % 3, (phase >> (g.nt % 3)) & 1u)) failed = true;
        phase ^= 1u << (g.nt % 3);
        __syncthreads();
        cl_sync();

        for (int t = g.nt - 1; t >= 0; --t) {
            const float* cb = ((t + 1) & 1) ? M1 : M0;   // a * lambda_{t+3}
            float* nb = (t & 1) ? M1 : M0;               // a * lambda_{t+2}
            const unsigned nb_addr = (t & 1) ? addr1 : addr0;
            // refill the buffer of level t+2 (last read at step t+1) with level t-1
            if (tid == 0 && t >= 1) {
                const int q = (t - 1) % 3;
                fence_proxy_async();
                mbar_expect_tx(bars + q, band_bytes);
                tma_load_1d(U + q * band, hist + (long long)(t - 1) * g.NP, band_bytes, bars + q);
            }
            const int b1 = t % 3, b2 = (t + 1) % 3;
            if (!mbar_wait_bounded(bars + b1, (phase >> b1) & 1u)) failed = true;
            phase ^= 1u << b1;
            const float* U1 = U + b1 * band;   // u_{t+1}
            const float* U2 = U + b2 * band;   // u_{t+2}
            if (live) {
                if (warp_seed) {
                    if (full)
                        adj_strip<RPT, SP, true, true>(cb, nb, A, OM, U1, U2, lam, mu, gv, gk, r_begin, nrows, x, j0,
                                                        s0, j1, s1);
                    else
                        adj_strip<RPT, SP, false, true>(cb, nb, A, OM, U1, U2, lam, mu, gv, gk, r_begin, nrows, x, j0,
                                                         s0, j1, s1);
                } else {
                    if (full)
                        adj_strip<RPT, SP, true, false>(cb, nb, A, OM, U1, U2, lam, mu, gv, gk, r_begin, nrows, x, -1,
                                                         0.0f, -1, 0.0f);
                    else
                        adj_strip<RPT, SP, false, false>(cb, nb, A, OM, U1, U2, lam, mu, gv, gk, r_begin, nrows, x, -1,
                                                          0.0f, -1, 0.0f);
                }
                push_edges<SP>(nb, nb_addr, b, r_begin, nrows, x);
            }
            cl_arrive();
            // next step's seeds load while the cluster meets
            if (t >= 1) {
                if (j0 >= 0) s0 = __ldg(seed + (long long)(t - 1) * g.nrec + r0);
                if (j1 >= 0) s1 = __ldg(seed + (long long)(t - 1) * g.nrec + r1);
            }
            cl_wait();
        }
        if (live) {
            float* gvo = a.gv + (long long)slot * g.NP + (long long)(b.z0 + r_begin) * g.pitch + x;
            float* gko = a.gk + (long long)slot * g.NP + (long long)(b.z0 + r_begin) * g.pitch + x;
#pragma unroll
            for (int j = 0; j < RPT; ++j)
                if (j < nrows) {
                    gvo[j * SP] = gv[j];
                    gko[j * SP] = gk[j];
                }
        }
        __syncthreads();
    }
    if (failed) atomicOr(a.err, 1);
}

}  // namespace
}  // namespace seis
