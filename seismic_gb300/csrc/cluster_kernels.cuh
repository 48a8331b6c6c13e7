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
//      distributed shared memory (mapa + st.async), each push counted on the
//      receiving CTA's mbarrier of that buffer (complete_tx bytes),
//   3. meets its own threads at one __syncthreads.
// There is no cluster-wide barrier per step: before reading a buffer a CTA
// waits (bounded) on that buffer's halo mbarrier only.  Neighbours then run at
// most one step apart, and with three wavefield buffers the buffer a CTA
// writes (and its neighbours push into) is never one that a neighbour may
// still be reading.
// Each thread owns one column x (or a column pair x, x+1: W = 2) and a strip
// of RPT consecutive rows of its band; it walks the strip with a 5-row sliding
// window in registers (vertical neighbours), reads the horizontal neighbours
// from shared memory at compile-time row offsets (the row pitch SP is a
// template parameter) plus per-thread column offsets that already carry the
// periodic wrap in x (so the edge columns cost no extra work), and keeps its
// per-point private state (the increments u, or the adjoint's lambda, mu and
// gradient sums) in registers.  Work that concerns few points -- halo pushes,
// the source, receiver gathers and seeds -- runs outside the point loop or in
// warp-uniform variants of the time loop, which is specialised per thread
// variant and chosen once per shot, so the common warps run a lean loop.
//
// The adjoint additionally streams the forward increments u_{t+1}, u_{t+2}
// of its band back from HBM with 1-D TMA bulk copies (cp.async.bulk +
// mbarrier complete_tx) into a 3-deep shared-memory ring, one step ahead of
// use.  In the adjoint one thread waits for the next step's halo rows and
// history level at the end of a step and the step's closing __syncthreads
// publishes them (the other threads issue no waits); in the forward the
// threads of the strips that read halo rows (within two rows of a band edge)
// wait for every phase of them and the interior strips never wait.  Every mbarrier wait is bounded: on timeout the kernel records an error
// in the error word (1: history copy, 2: a copy still pending at exit, 4: halo
// rows), stops waiting on that kind of barrier, still meets the cluster
// barriers between shots (so no CTA is left waiting), and the host reports it.
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
__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ unsigned cl_map(unsigned local_addr, unsigned rank)
{
    unsigned r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(local_addr), "r"(rank));
    return r;
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
    // tangent (forward sweeps with TAN)
    const float* alpha_d;  // [model][NP]
    const float* kdfac;    // [model] min_vel_diff * dt
    const float* smod_d;   // [slot][nt]
    float* drec;           // [slot][nt][nrec]
    float* uhist;          // [slot][nt+1][NP] (forward writes levels 1..nt, adjoint reads)
    long long u_slot_stride;
    int write_hist;
    // adjoint
    const float* seed;     // [slot][nt][nrec]
    float* gv;             // [slot][NP]
    float* gk;             // [slot][NP]
    int* err;              // error word: 1 = an mbarrier wait timed out
    int skip_copy_level;   // test hook: this history level is never copied (its wait must time out); -1 = none
};

__device__ __forceinline__ int band_rows(int k, int R, int NZ)
{
    const int r = NZ - k * R;
    return r < R ? r : R;
}

// A compile-time bool as a value (selects a specialised time loop).
template <bool B>
struct integral_c {
    static constexpr bool value = B;
};

// Per-CTA constants of a band: wavefield buffers are [R+4][SP] with band row
// r at buffer row r+2 and column x at buffer column x+2.
template <int SP>
struct Band {
    int k, Rk, R_up, z0, NX;
    unsigned up_rank, dn_rank;
    __device__ __forceinline__ static int at(int r, int x) { return (r + 2) * SP + x + 2; }
};

// One strip of one thread: rows [r_begin, r_begin + nrows) of the band, walked
// downwards, or upwards (UP) by the last strip of the CTA so that both the
// CTA's first two rows (first strip) and its last two rows (last strip) are
// computed first and pushed to the neighbours early in the step.
struct Strip {
    int r_begin, nrows;
    bool push_top;     // this strip computes rows 0,1 first and pushes them up inline
    bool push_bottom;  // this strip computes rows Rk-1,Rk-2 first and pushes them down inline
};

// W consecutive columns of one row (W = 1 or 2) held as one value, float or
// float2, loaded and stored as one 4- or 8-byte access (W = 2 needs an even
// column index, which holds for every buffer index at(r, x) with x even since SP
// is even).  Column pairs are computed with packed FP32 instructions (add2 /
// mul2 / fma2), each lane rounded as the scalar operation.
template <int W>
struct VecT {
    using type = float;
};
template <>
struct VecT<2> {
    using type = float2;
};
template <int W>
using Vec = typename VecT<W>::type;

__device__ __forceinline__ float vadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float2 vadd(float2 a, float2 b) { return add2(a, b); }
__device__ __forceinline__ float vmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float2 vmul(float2 a, float2 b) { return mul2(a, b); }
__device__ __forceinline__ float vfma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ float2 vfma(float2 a, float2 b, float2 c) { return fma2(a, b, c); }
__device__ __forceinline__ float vneg(float a) { return -a; }
__device__ __forceinline__ float2 vneg(float2 a) { return make_float2(-a.x, -a.y); }
template <int W>
__device__ __forceinline__ Vec<W> vsplat(float a)
{
    if constexpr (W == 2) return make_float2(a, a);
    else return a;
}
// lane w of v += s (one column of the pair: the source or a receiver seed)
template <int W>
__device__ __forceinline__ void add_lane(Vec<W>& v, int w, float s)
{
    if constexpr (W == 2) {
        if (w) v.y += s;
        else v.x += s;
    } else {
        v += s;
    }
}

template <int W>
__device__ __forceinline__ Vec<W> ld_cols(const float* p)
{
    if constexpr (W == 2) return *reinterpret_cast<const float2*>(p);
    else return *p;
}
template <int W>
__device__ __forceinline__ void st_cols(float* p, const Vec<W>& c)
{
    if constexpr (W == 2) *reinterpret_cast<float2*>(p) = c;
    else *p = c;
}
// Asynchronous store of W floats into a neighbour's shared memory whose bytes
// are counted on the neighbour's mbarrier (complete_tx): the neighbour reads
// them only after that barrier's phase completes.
template <int W>
__device__ __forceinline__ void st_async_cols(unsigned cluster_addr, unsigned cluster_bar, const Vec<W>& c)
{
    if constexpr (W == 2)
        asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v2.f32 [%0], {%1, %2}, [%3];" ::"r"(
                         cluster_addr),
                     "f"(c.x), "f"(c.y), "r"(cluster_bar)
                     : "memory");
    else
        asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.f32 [%0], %1, [%2];" ::"r"(cluster_addr),
                     "f"(c), "r"(cluster_bar)
                     : "memory");
}

// Where a step's halo rows go: the shared addresses of the buffer the step
// writes and of that buffer's halo mbarrier (the same offsets in every CTA).
struct HaloDst {
    unsigned buf;
    unsigned bar;
};

// Push of band row r (columns x .. x+W-1) into the halo rows of the
// neighbour above (its rows R_up, R_up + 1) or below (its rows -2, -1).
template <int SP, int W>
__device__ __forceinline__ void push_up_cols(const HaloDst& h, const Band<SP>& b, int r, int x, const Vec<W>& v)
{
    st_async_cols<W>(cl_map(h.buf + 4u * (unsigned)Band<SP>::at(b.R_up + r, x), b.up_rank), cl_map(h.bar, b.up_rank),
                     v);
}
template <int SP, int W>
__device__ __forceinline__ void push_down_cols(const HaloDst& h, const Band<SP>& b, int r, int x, const Vec<W>& v)
{
    st_async_cols<W>(cl_map(h.buf + 4u * (unsigned)Band<SP>::at(r - b.Rk, x), b.dn_rank), cl_map(h.bar, b.dn_rank),
                     v);
}

// Where a thread finds the horizontal neighbours of its W columns within a
// row: offsets in floats from its first column x, wrapped periodically in x as
// in the reference (core/seis_forward2.py:395-403).  W = 2: the pair of columns
// x-2, x-1 at xl and the pair x+2, x+3 at xr (NX even, so a pair never
// straddles the wrap); W = 1: columns x-2, x-1, x+1, x+2 at o[0..3].
template <int W>
struct XWrap {
    int o[W == 2 ? 2 : 4];
};
template <int W>
__device__ __forceinline__ XWrap<W> make_xwrap(int x, int NX)
{
    auto wrap = [NX](int c) { return c < 0 ? c + NX : (c >= NX ? c - NX : c); };
    XWrap<W> xw;
    if constexpr (W == 2) {
        xw.o[0] = wrap(x - 2) - x;
        xw.o[1] = wrap(x + 2) - x;
    } else {
        xw.o[0] = wrap(x - 2) - x;
        xw.o[1] = wrap(x - 1) - x;
        xw.o[2] = wrap(x + 1) - x;
        xw.o[3] = wrap(x + 2) - x;
    }
    return xw;
}
// Horizontal neighbour sums of the thread's W columns in one row (row points at
// column x; c the thread's own values): h1 = (x+1) + (x-1) and h2 = (x+2) + (x-2)
// per column, in that order.
template <int W>
__device__ __forceinline__ void horiz_sums(const float* row, const XWrap<W>& xw, const Vec<W>& c, Vec<W>& h1,
                                           Vec<W>& h2)
{
    if constexpr (W == 2) {
        const float2 l = *reinterpret_cast<const float2*>(row + xw.o[0]);   // columns x-2, x-1
        const float2 r = *reinterpret_cast<const float2*>(row + xw.o[1]);   // columns x+2, x+3
        h1 = make_float2(c.y + l.y, r.x + c.x);
        h2 = add2(r, l);
    } else {
        h1 = row[xw.o[2]] + row[xw.o[1]];
        h2 = row[xw.o[3]] + row[xw.o[0]];
    }
}

// The same sums with the neighbour pairs taken from the adjacent lanes by warp
// shuffles (W = 2: lane l - 1 holds columns x-2, x-1 and lane l + 1 holds x+2, x+3
// in its own pair); shared loads remain for the lanes whose neighbour is not the
// adjacent lane (lane 0 and 31, the periodic wrap, a neighbour past the grid).
// `mask` holds the warp's live lanes, which execute every shuffle together.
struct LaneNbr {
    unsigned mask;
    bool fix_l, fix_r;
};
__device__ __forceinline__ void horiz_sums_shfl(const float* row, const XWrap<2>& xw, const float2& c,
                                                const LaneNbr& ln, float2& h1, float2& h2)
{
    float lx = __shfl_up_sync(ln.mask, c.x, 1), ly = __shfl_up_sync(ln.mask, c.y, 1);
    float rx = __shfl_down_sync(ln.mask, c.x, 1), ry = __shfl_down_sync(ln.mask, c.y, 1);
    if (ln.fix_l) {
        const float2 l = *reinterpret_cast<const float2*>(row + xw.o[0]);
        lx = l.x;
        ly = l.y;
    }
    if (ln.fix_r) {
        const float2 r = *reinterpret_cast<const float2*>(row + xw.o[1]);
        rx = r.x;
        ry = r.y;
    }
    h1 = make_float2(c.y + ly, rx + c.x);
    h2 = add2(make_float2(rx, ry), make_float2(lx, ly));
}

// A thread's edge duties, fixed for the whole sweep, packed in one word:
// bit q / 4 + q: push band row (q < 2 ? q : Rk - 4 + q) up / down because the
// strip does not push it inline (short bands).
template <int SP, int W>
__device__ __forceinline__ unsigned edge_work(const Band<SP>& b, const Strip& s, int x)
{
    unsigned e = 0u;
    const int r_end = s.r_begin + s.nrows;
    for (int q = 0; q < 4; ++q) {
        const int r = q < 2 ? q : b.Rk - 4 + q;
        if (r < s.r_begin || r >= r_end || (q >= 2 && r < 2)) continue;
        if (q < 2 && !s.push_top) e |= 1u << q;
        if (r >= b.Rk - 2 && !s.push_bottom) e |= 1u << (4 + q);
    }
    return e;
}

// After the strip: the thread's edge duties (edge_work).  Reads back the
// values this thread just wrote; x is the first of the thread's W columns.
template <int SP, int W>
__device__ __forceinline__ void finish_edges(float* nb, const HaloDst& hd, const Band<SP>& b, const Strip& s, int x,
                                             unsigned e)
{
    if (!e) return;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        if (!((e >> q) & 0x11u)) continue;
        const int r = q < 2 ? q : b.Rk - 4 + q;
        const Vec<W> v = ld_cols<W>(nb + Band<SP>::at(r, x));
        if ((e >> q) & 1u) push_up_cols<SP, W>(hd, b, r, x, v);
        if ((e >> (4 + q)) & 1u) push_down_cols<SP, W>(hd, b, r, x, v);
    }
}

// 1 - kappa over a thread's strip, held as the sponge profile is built
// (core/seis_forward2.py:46-59): in the side bands (x outside the interior
// columns) it depends on the column only, elsewhere on the row only.
template <int RPT, int W>
struct OneMinusKappa {
    float row[RPT];   // walk row j, interior columns
    float col[W];     // column x + w, side bands
    unsigned side;    // bit w: column x + w lies in a side band
    __device__ __forceinline__ Vec<W> at(int j) const
    {
        if constexpr (W == 2) return make_float2((side & 1u) ? col[0] : row[j], (side & 2u) ? col[1] : row[j]);
        else return (side & 1u) ? col[0] : row[j];
    }
};

// Strip of the forward step: u' = (1-k) u + a Lap(p) [+ src], p' = p + u'.
// Each thread owns W adjacent columns x .. x+W-1 (W = 1 or 2) of its strip.
// FULL: the strip has RPT rows; SRC: the strip may hold the source (row jsrc of
// the walk, column x + scol); UP: walk upwards.  The stencil's sum order is the
// same for every W and both directions, so all variants give bitwise equal results.
template <int RPT, int W, int SP, bool AS, bool FULL, bool SRC, bool UP, bool SH>
__device__ __forceinline__ void fwd_strip(const float* __restrict__ cb, float* __restrict__ nb, const HaloDst& hd,
                                          const Band<SP>& b, const Vec<W> (&a)[AS ? 1 : RPT],
                                          const float* __restrict__ A, const OneMinusKappa<RPT, W>& om,
                                          Vec<W> (&u)[RPT], const Strip& s, int x, const XWrap<W>& xw, int jsrc,
                                          int scol, float src, const LaneNbr& ln)
{
    // first row walked: r0; direction d; buffer row of band row r is r + 2
    const int r0 = UP ? s.r_begin + s.nrows - 1 : s.r_begin;
    constexpr int D = UP ? -1 : 1;
    const float* col = cb + (r0 + 2) * SP + x + 2;      // band row r0, column x
    Vec<W> w0 = ld_cols<W>(col - 2 * D * SP), w1 = ld_cols<W>(col - D * SP), w2 = ld_cols<W>(col),
           w3 = ld_cols<W>(col + D * SP);
    float* out = nb + (r0 + 2) * SP + x + 2;
    const float* arow = A + r0 * SP + x;
#pragma unroll
    for (int j = 0; j < RPT; ++j) {
        if (FULL || j < s.nrows) {
            const Vec<W> w4 = ld_cols<W>(col + (j + 2) * D * SP);   // band row r0 + (j+2) D
            Vec<W> av;
            if constexpr (AS) av = ld_cols<W>(arow + j * D * SP);
            else av = a[j];
            Vec<W> h1, h2;
            if constexpr (SH && W == 2) horiz_sums_shfl(col + j * D * SP, xw, w2, ln, h1, h2);
            else horiz_sums<W>(col + j * D * SP, xw, w2, h1, h2);
            // (east + west) + (row below + row above); (+-2 likewise)
            const Vec<W> t1 = vadd(h1, vadd(w3, w1)), t2 = vadd(h2, vadd(w4, w0));
            Vec<W> un = fwd_increment(om.at(j), u[j], av, stencil_lap(w2, t1, t2));
            if (SRC && j == jsrc) add_lane<W>(un, scol, src);
            u[j] = un;
            const Vec<W> pn = vadd(w2, un);
            st_cols<W>(out + j * D * SP, pn);
            if (j < 2) {
                if (!UP && s.push_top) push_up_cols<SP, W>(hd, b, s.r_begin + j, x, pn);
                if (UP && s.push_bottom) push_down_cols<SP, W>(hd, b, r0 - j, x, pn);
            }
            w0 = w1; w1 = w2; w2 = w3; w3 = w4;
        }
    }
}

// Strip of the forward + tangent step (the tiled fwd_step_kernel<true>'s
// arithmetic): u' and p' as in fwd_strip, and
//   du' = (1-k) du + a Lap(dp) + a_d Lap(p) - k_d u [+ src_d],  dp' = dp + du'
// with a_d = dalpha (shared memory) and nk = -k_d (registers).  Both fields'
// edge rows are pushed (hd: p buffer, hdd: dp buffer, same barrier).
template <int RPT, int W, int SP, bool AS, bool FULL, bool SRC, bool UP>
__device__ __forceinline__ void tan_strip(const float* __restrict__ cb, float* __restrict__ nb,
                                          const float* __restrict__ dcb, float* __restrict__ dnb, const HaloDst& hd,
                                          const HaloDst& hdd, const Band<SP>& b, const Vec<W> (&a)[AS ? 1 : RPT],
                                          const float* __restrict__ A, const float* __restrict__ AD,
                                          const OneMinusKappa<RPT, W>& om, const OneMinusKappa<RPT, W>& nk,
                                          Vec<W> (&u)[RPT], Vec<W> (&du)[RPT], const Strip& s, int x,
                                          const XWrap<W>& xw, int jsrc, int scol, float src, float src_d)
{
    const int r0 = UP ? s.r_begin + s.nrows - 1 : s.r_begin;
    constexpr int D = UP ? -1 : 1;
    const int c0 = (r0 + 2) * SP + x + 2;                  // buffer offset of band row r0, column x
    const float* col = cb + c0;
    const float* dcol = dcb + c0;
    Vec<W> w0 = ld_cols<W>(col - 2 * D * SP), w1 = ld_cols<W>(col - D * SP), w2 = ld_cols<W>(col),
           w3 = ld_cols<W>(col + D * SP);
    Vec<W> v0 = ld_cols<W>(dcol - 2 * D * SP), v1 = ld_cols<W>(dcol - D * SP), v2 = ld_cols<W>(dcol),
           v3 = ld_cols<W>(dcol + D * SP);
    const int a0 = r0 * SP + x;
#pragma unroll
    for (int j = 0; j < RPT; ++j) {
        if (FULL || j < s.nrows) {
            const Vec<W> w4 = ld_cols<W>(col + (j + 2) * D * SP);
            const Vec<W> v4 = ld_cols<W>(dcol + (j + 2) * D * SP);
            Vec<W> av;
            if constexpr (AS) av = ld_cols<W>(A + a0 + j * D * SP);
            else av = a[j];
            const Vec<W> adv = ld_cols<W>(AD + a0 + j * D * SP);
            Vec<W> h1, h2, g1, g2;
            horiz_sums<W>(col + j * D * SP, xw, w2, h1, h2);
            horiz_sums<W>(dcol + j * D * SP, xw, v2, g1, g2);
            const Vec<W> t1 = vadd(h1, vadd(w3, w1)), t2 = vadd(h2, vadd(w4, w0));
            const Vec<W> d1 = vadd(g1, vadd(v3, v1)), d2 = vadd(g2, vadd(v4, v0));
            const Vec<W> L = stencil_lap(w2, t1, t2);
            const Vec<W> dL = stencil_lap(v2, d1, d2);
            const Vec<W> omw = om.at(j);
            Vec<W> un = fwd_increment(omw, u[j], av, L);
            Vec<W> dun;
            if constexpr (W == 2) {
                const float2 nkw = nk.at(j);
                dun.x = tan_increment_nkd(omw.x, du[j].x, av.x, dL.x, adv.x, L.x, nkw.x, u[j].x);
                dun.y = tan_increment_nkd(omw.y, du[j].y, av.y, dL.y, adv.y, L.y, nkw.y, u[j].y);
            } else {
                dun = tan_increment_nkd(omw, du[j], av, dL, adv, L, nk.at(j), u[j]);
            }
            if (SRC && j == jsrc) {
                add_lane<W>(un, scol, src);
                add_lane<W>(dun, scol, src_d);
            }
            u[j] = un;
            du[j] = dun;
            const Vec<W> pn = vadd(w2, un), dpn = vadd(v2, dun);
            st_cols<W>(nb + c0 + j * D * SP, pn);
            st_cols<W>(dnb + c0 + j * D * SP, dpn);
            if (j < 2) {
                if (!UP && s.push_top) {
                    push_up_cols<SP, W>(hd, b, s.r_begin + j, x, pn);
                    push_up_cols<SP, W>(hdd, b, s.r_begin + j, x, dpn);
                }
                if (UP && s.push_bottom) {
                    push_down_cols<SP, W>(hd, b, r0 - j, x, pn);
                    push_down_cols<SP, W>(hdd, b, r0 - j, x, dpn);
                }
            }
            w0 = w1; w1 = w2; w2 = w3; w3 = w4;
            v0 = v1; v1 = v2; v2 = v3; v3 = v4;
        }
    }
}

// The strip's increments u[j] (band row r0 + j D) into one history level;
// hp points at the walk's first row.
template <int RPT, int W, int SP, bool FULL, bool UP>
__device__ __forceinline__ void store_hist(float* __restrict__ hp, const Vec<W> (&u)[RPT], int nrows)
{
    constexpr int D = UP ? -1 : 1;
#pragma unroll
    for (int j = 0; j < RPT; ++j)
        if (FULL || j < nrows) st_cols<W>(hp + j * D * SP, u[j]);
}

// ---------------------------------------------------------------------------
// forward sweep
// smem: P[3][R+4][SP] | DP[3][R+4][SP] (TAN) | A[R][SP] (alpha, AS) | AD[R][SP] (dalpha, TAN) |
//       halo mbar[3] | S[nt] | SD[nt] (TAN) | receivers of the band (3 x nrec ints) | count.
// alpha and 1-kappa of a thread's strip stay in its registers for the sweep.
// ---------------------------------------------------------------------------
template <int SP>
__device__ __forceinline__ Strip make_strip(const Band<SP>& b, int gg, int G, int RPT)
{
    Strip s;
    s.r_begin = gg * RPT;
    s.nrows = max(0, min(RPT, b.Rk - s.r_begin));
    const bool up = gg == G - 1 && G > 1;
    s.push_top = !up && s.r_begin == 0 && s.nrows >= 2;
    s.push_bottom = up && s.r_begin + s.nrows == b.Rk && s.nrows >= 2;
    return s;
}

// W columns per thread (1, or 2 for an even NX): the thread groups of SP / W
// threads each cover one strip of RPT rows across the whole band width.  AS:
// alpha of the band in shared memory (frees RPT * W registers per thread for
// the longer strips), else in registers.  TAN: the tangent (Born) field
// advances beside the wavefield (dp buffers, dalpha in shared memory, dkappa
// and du in registers) and its records go to a.drec.
template <int C, int RPT, int W, int SP, int NTHR, bool AS, bool TAN, bool SH = false>
__global__ void __launch_bounds__(NTHR, 1) fwd_cluster_kernel(ClusterArgs a)
{
    constexpr int GW = SP / W;   // threads per strip group
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
    float* P = sm;                         // 3 buffers: p_m in buffer m % 3
    float* DP = P + 3 * bufsz;             // 3 buffers of dp (TAN only)
    float* A = DP + (TAN ? 3 * bufsz : 0); // alpha of the band [R][SP] (AS only)
    float* AD = A + (AS ? R * SP : 0);     // dalpha of the band [R][SP] (TAN only)
    uint64_t* hb = (uint64_t*)(AD + (TAN ? R * SP : 0));   // halo mbarrier of each buffer
    float* SRC = (float*)(hb + 3);
    float* SRCD = SRC + g.nt;              // tangent source series (TAN only)
    int* RL = (int*)(SRCD + (TAN ? g.nt : 0));   // [3][nrec]: band row, column, receiver id
    int* nrl = RL + 3 * g.nrec;
    const int tid = threadIdx.x;
    const int x = W * (tid % GW), gg = tid / GW;   // first column of the thread, strip group
    const Strip st = make_strip<SP>(b, gg, a.G, RPT);
    const bool up = gg == a.G - 1 && a.G > 1;
    const bool live = x < g.NX && st.nrows > 0;      // W = 2 needs NX even: both columns live
    LaneNbr ln{};                                    // neighbour shuffles (SH)
    if constexpr (SH) {
        const unsigned lane = threadIdx.x & 31u;
        ln.mask = __ballot_sync(0xffffffffu, live);
        ln.fix_l = lane == 0 || x - 2 < 0;
        ln.fix_r = lane == 31 || !((ln.mask >> (lane + 1)) & 1u) || x + 2 + W > g.NX;
    }
    const bool full = st.nrows == RPT;
    const unsigned ew = edge_work<SP, W>(b, st, x);
    const XWrap<W> xw = make_xwrap<W>(x, g.NX);
    const unsigned halo_bytes = (TAN ? 32u : 16u) * (unsigned)g.NX;   // two rows of each field from each neighbour
    unsigned hphase = 0u;       // bit k: parity of the next phase to wait for on hb[k]
    bool halo_failed = false;
    // only strips whose stencil reaches a halo row (within two rows of a band edge)
    // wait for the halo rows, every phase of them (their parities stay exact); the
    // others never wait
    const bool reads_halo = tid == 0 || st.r_begin < 2 || st.r_begin + st.nrows + 2 > b.Rk;
    if (tid == 0) {
        for (int k = 0; k < 3; ++k) mbar_init(hb + k, 1);
        fence_mbar_init();
    }
    // p_m's halo rows, pushed by the neighbours in their step m-2 (bounded wait)
    auto wait_halo = [&](int k) {
        if (!halo_failed && !mbar_wait_bounded(hb + k, (hphase >> k) & 1u)) halo_failed = true;
        hphase ^= 1u << k;
    };

    for (int slot = (int)cl_id(); slot < a.slots; slot += (int)cl_count()) {
        const ShotDesc sd = a.shots[slot];
        if (!sd.active) break;  // uniform across the cluster
        const float* al = a.alpha + (long long)sd.model * g.NP;
        const float kf = __ldg(a.kfac + sd.model);
        if (tid == 0) *nrl = 0;
        for (int i = tid; i < (TAN ? 6 : 3) * bufsz; i += blockDim.x) sm[i] = 0.0f;
        // alpha and 1-kappa of this thread's strip, in walk order
        if (AS)
            for (int i = tid; i < b.Rk * SP; i += blockDim.x) {
                const int r = i / SP, xx = i - r * SP;
                A[i] = xx < g.NX ? __ldg(al + (long long)(b.z0 + r) * g.pitch + xx) : 0.0f;
            }
        if (TAN) {
            const float* ald = a.alpha_d + (long long)sd.model * g.NP;
            for (int i = tid; i < b.Rk * SP; i += blockDim.x) {
                const int r = i / SP, xx = i - r * SP;
                AD[i] = xx < g.NX ? __ldg(ald + (long long)(b.z0 + r) * g.pitch + xx) : 0.0f;
            }
        }
        Vec<W> ar[AS ? 1 : RPT];
        OneMinusKappa<RPT, W> omr, kdr;   // 1 - kappa and (TAN) -dkappa over the strip
        {
            const int r0 = up ? st.r_begin + st.nrows - 1 : st.r_begin;
            const float kdf = TAN ? __ldg(a.kdfac + sd.model) : 0.0f;
            omr.side = 0u;
#pragma unroll
            for (int w = 0; w < W; ++w) {
                const int xc = x + w;
                const bool side = xc < g.xlo || xc >= g.xhi;
                omr.side |= (unsigned)side << w;
                omr.col[w] = live && side ? one_minus_kappa_of(kf, __ldg(a.dampx + xc)) : 0.0f;
                kdr.col[w] = TAN && live && side ? -__fmul_rn(kdf, __ldg(a.dampx + xc)) : 0.0f;
            }
            kdr.side = omr.side;
#pragma unroll
            for (int j = 0; j < RPT; ++j) {
                const int z = b.z0 + (up ? r0 - j : r0 + j);
                const bool in = live && j < st.nrows;
                omr.row[j] = in ? one_minus_kappa_of(kf, __ldg(a.dampz + z)) : 0.0f;
                kdr.row[j] = TAN && in ? -__fmul_rn(kdf, __ldg(a.dampz + z)) : 0.0f;
                if (!AS) {
                    float av[W];
#pragma unroll
                    for (int w = 0; w < W; ++w) av[w] = in ? __ldg(al + (long long)z * g.pitch + x + w) : 0.0f;
                    if constexpr (W == 2) ar[AS ? 0 : j] = make_float2(av[0], av[1]);
                    else ar[AS ? 0 : j] = av[0];
                }
            }
        }
        const float* smod = a.smod + (long long)slot * g.nt;
        for (int i = tid; i < g.nt; i += blockDim.x) SRC[i] = __ldg(smod + i);
        if (TAN) {
            const float* smd = a.smod_d + (long long)slot * g.nt;
            for (int i = tid; i < g.nt; i += blockDim.x) SRCD[i] = __ldg(smd + i);
        }
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
        // the source, as an index along this thread's walk
        const int sz = sd.src_off / g.pitch - b.z0, sx = sd.src_off % g.pitch;
        int jsrc = -1;
        const int scol = sx - x;
        if (live && scol >= 0 && scol < W && sz >= st.r_begin && sz < st.r_begin + st.nrows)
            jsrc = up ? st.r_begin + st.nrows - 1 - sz : sz - st.r_begin;
        const bool warp_src = __any_sync(0xffffffffu, jsrc >= 0);
        float* rec = a.rec + (long long)slot * g.nt * g.nrec;
        // history level 1 at this thread's first walk row (levels are NP apart)
        float* hist = a.write_hist ? a.uhist + (long long)slot * a.u_slot_stride + (long long)b.z0 * g.pitch + x
                                   : nullptr;
        Vec<W> u[RPT], du[TAN ? RPT : 1];
#pragma unroll
        for (int j = 0; j < RPT; ++j) {
            u[j] = vsplat<W>(0.0f);
            if (TAN) du[TAN ? j : 0] = vsplat<W>(0.0f);
        }
        float* drec = TAN ? a.drec + (long long)slot * g.nt * g.nrec : nullptr;
        __syncthreads();
        const int nr = *nrl;
        // the gather runs on the second strip group (no halo waits or pushes there)
        const int gather0 = a.G > 2 ? (int)blockDim.x / a.G : 0;
        cl_sync();   // every CTA's buffers are clear (and its barriers ready) before the first push

        // Step t reads p_{t+1} and writes p_{t+2}.  No cluster-wide barrier per
        // step: a CTA waits only for its halo rows, and the neighbours can run at
        // most one step apart, so three buffers keep every buffer that a
        // neighbour may still push into or read distinct from the ones in use.
        // The time loop, specialised per thread variant (walk direction, full
        // strip, source in the warp) so that the loop-carried registers stay put;
        // the variant is chosen once per slot.  Returns the buffer of p_{nt+1}.
        auto time_loop = [&](auto full_c, auto src_c, auto up_c) {
            constexpr bool F = decltype(full_c)::value, S = decltype(src_c)::value, U = decltype(up_c)::value;
            const long long hrow = (long long)(U ? st.r_begin + st.nrows - 1 : st.r_begin) * SP;
            int kc = 1;   // buffer of p_{t+1}: (t+1) % 3; p_{t+2} is in the next one
            for (int t = 0; t < g.nt; ++t) {
                const int kn = kc == 2 ? 0 : kc + 1;
                const float* cb = P + kc * bufsz;
                float* nb = P + kn * bufsz;
                const float* dcb = DP + kc * bufsz;
                float* dnb = DP + kn * bufsz;
                const HaloDst hd{smem_addr(nb), smem_addr(hb + kn)};
                const HaloDst hdd{smem_addr(dnb), hd.bar};
                if (tid == 0) mbar_expect_tx(hb + kn, halo_bytes);
                if (t > 0) {
                    if (reads_halo) wait_halo(kc);
                    // record row t-1 = p_{t+1}, complete in this CTA's buffer
                    for (int i = tid - gather0; i >= 0 && i < nr; i += blockDim.x) {
                        const int bo = Band<SP>::at(RL[i], RL[g.nrec + i]);
                        const long long ro = (long long)(t - 1) * g.nrec + RL[2 * g.nrec + i];
                        rec[ro] = cb[bo];
                        if (TAN) drec[ro] = dcb[bo];
                    }
                }
                if (live) {
                    if constexpr (TAN) {
                        tan_strip<RPT, W, SP, AS, F, S, U>(cb, nb, dcb, dnb, hd, hdd, b, ar, A, AD, omr, kdr, u, du,
                                                           st, x, xw, jsrc, scol, SRC[t], SRCD[t]);
                        finish_edges<SP, W>(dnb, hdd, b, st, x, ew);
                    } else {
                        fwd_strip<RPT, W, SP, AS, F, S, U, SH>(cb, nb, hd, b, ar, A, omr, u, st, x, xw, jsrc, scol,
                                                               SRC[t], ln);
                    }
                    finish_edges<SP, W>(nb, hd, b, st, x, ew);
                    if (hist) store_hist<RPT, W, SP, F, U>(hist + (long long)(t + 1) * g.NP + hrow, u, st.nrows);
                }
                __syncthreads();
                kc = kn;
            }
            return kc;
        };
        using Yes = integral_c<true>;
        using No = integral_c<false>;
        int kc;
        if (up) {
            if (warp_src) kc = full ? time_loop(Yes{}, Yes{}, Yes{}) : time_loop(No{}, Yes{}, Yes{});
            else kc = full ? time_loop(Yes{}, No{}, Yes{}) : time_loop(No{}, No{}, Yes{});
        } else {
            if (warp_src) kc = full ? time_loop(Yes{}, Yes{}, No{}) : time_loop(No{}, Yes{}, No{});
            else kc = full ? time_loop(Yes{}, No{}, No{}) : time_loop(No{}, No{}, No{});
        }
        if (reads_halo) wait_halo(kc);   // p_{nt+1}'s halo rows (not read) have all landed
        // last record row: p_{nt+1}
        const float* fb = P + kc * bufsz;
        for (int i = tid; i < nr; i += blockDim.x) {
            const int bo = Band<SP>::at(RL[i], RL[g.nrec + i]);
            const long long ro = (long long)(g.nt - 1) * g.nrec + RL[2 * g.nrec + i];
            rec[ro] = fb[bo];
            if (TAN) drec[ro] = DP[kc * bufsz + bo];
        }
        cl_sync();   // every CTA done with its buffers before the next slot clears them
    }
    if (halo_failed) atomicOr(a.err, 4);
}

// Strip of the adjoint step (UP: walk upwards; same sum order both ways):
//   mu = (1-k) mu + Lap(a lambda') [+ seed],  lambda = lambda' + mu,
//   Gv += lambda (u_{t+2} - (1-k) u_{t+1}),  Gk += lambda u_{t+1},  M' = a lambda.
// Each thread owns W adjacent columns from x; the seeds s0, s1 enter at walk
// rows j0, j1 and columns x + c0, x + c1.  Every rounding step is written out,
// so all W and both directions agree bitwise.
template <int RPT, int W, int SP, bool FULL, bool SEED, bool UP>
__device__ __forceinline__ void adj_strip(const float* __restrict__ cb, float* __restrict__ nb, const HaloDst& hd,
                                          const Band<SP>& b, const float* __restrict__ AO, const float* __restrict__ U1,
                                          const float* __restrict__ U2, Vec<W> (&lam)[RPT], Vec<W> (&mu)[RPT],
                                          Vec<W> (&gv)[RPT], Vec<W> (&gk)[RPT], const Strip& s, int x,
                                          const XWrap<W>& xw, int j0, int c0, float s0, int j1, int c1, float s1)
{
    const int r0 = UP ? s.r_begin + s.nrows - 1 : s.r_begin;
    constexpr int D = UP ? -1 : 1;
    const float* col = cb + (r0 + 2) * SP + x + 2;
    Vec<W> w0 = ld_cols<W>(col - 2 * D * SP), w1 = ld_cols<W>(col - D * SP), w2 = ld_cols<W>(col),
           w3 = ld_cols<W>(col + D * SP);
    const int o0 = r0 * SP + x;
    float* out = nb + (r0 + 2) * SP + x + 2;
#pragma unroll
    for (int j = 0; j < RPT; ++j) {
        if (FULL || j < s.nrows) {
            const Vec<W> w4 = ld_cols<W>(col + (j + 2) * D * SP);
            Vec<W> h1, h2;
            horiz_sums<W>(col + j * D * SP, xw, w2, h1, h2);
            const int o = o0 + j * D * SP;
            // alpha and 1-kappa of the thread's columns, interleaved: one 4W-byte load
            Vec<W> av, omv;
            if constexpr (W == 2) {
                const float4 q = *reinterpret_cast<const float4*>(AO + 2 * o);
                av = make_float2(q.x, q.y);
                omv = make_float2(q.z, q.w);
            } else {
                const float2 q = *reinterpret_cast<const float2*>(AO + 2 * o);
                av = q.x;
                omv = q.y;
            }
            const Vec<W> u1 = ld_cols<W>(U1 + o), u2 = ld_cols<W>(U2 + o);
            const Vec<W> t1 = vadd(h1, vadd(w3, w1)), t2 = vadd(h2, vadd(w4, w0));
            Vec<W> m = vfma(omv, mu[j], stencil_lap(w2, t1, t2));
            if (SEED) {
                if (j == j0) add_lane<W>(m, c0, s0);
                if (j == j1) add_lane<W>(m, c1, s1);
            }
            const Vec<W> lv = vadd(lam[j], m);
            mu[j] = m;
            lam[j] = lv;
            gv[j] = vfma(lv, vfma(vneg(omv), u1, u2), gv[j]);
            gk[j] = vfma(lv, u1, gk[j]);
            const Vec<W> mv = vmul(av, lv);
            st_cols<W>(out + j * D * SP, mv);
            if (j < 2) {
                if (!UP && s.push_top) push_up_cols<SP, W>(hd, b, s.r_begin + j, x, mv);
                if (UP && s.push_bottom) push_down_cols<SP, W>(hd, b, r0 - j, x, mv);
            }
            w0 = w1; w1 = w2; w2 = w3; w3 = w4;
        }
    }
}

// ---------------------------------------------------------------------------
// adjoint sweep (t = nt-1 .. 0)
// smem: M[3][R+4][SP] (a*lambda) | AO[R][SP][2] (alpha and 1-kappa interleaved per W columns) |
//       U[3][R][SP] | mbar[3] (history) |
//       mbar[3] (halos) | fail flag (8 B)
// ---------------------------------------------------------------------------
template <int C, int RPT, int W, int SP, int NTHR>
__global__ void __launch_bounds__(NTHR, 1) adj_cluster_kernel(ClusterArgs a)
{
    constexpr int GW = SP / W;   // threads per strip group
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
    float* M = sm;                                         // 3 buffers: a lambda_m in buffer m % 3
    float* A = sm + 3 * bufsz;
    float* AO = A;                                         // [R][SP / W][2][W]: alpha then 1-kappa
    float* U = A + 2 * band;                               // 3 levels of the band
    uint64_t* bars = (uint64_t*)(U + 3 * band);            // band*4 is a multiple of 128 bytes
    const int tid = threadIdx.x;
    const int x = W * (tid % GW), gg = tid / GW;
    const Strip st = make_strip<SP>(b, gg, a.G, RPT);
    const bool up = gg == a.G - 1 && a.G > 1;
    const bool live = x < g.NX && st.nrows > 0;
    const bool full = st.nrows == RPT;
    const unsigned band_bytes = (unsigned)(b.Rk * SP * 4);
    unsigned phase = 0u;    // bit i: parity of the next phase to wait for on barrier i
    unsigned pending = 0u;  // (thread 0) bit i: a copy on barrier i whose completion it has not seen
    bool failed = false;    // this thread gave up a wait, or saw another thread give up
    const unsigned ew = edge_work<SP, W>(b, st, x);
    const XWrap<W> xw = make_xwrap<W>(x, g.NX);
    uint64_t* hb = bars + 3;                               // halo mbarrier of each M buffer
    volatile int& s_fail = *(volatile int*)(bars + 6);   // 8 bytes after the 6 mbarriers
    const unsigned halo_bytes = 16u * (unsigned)g.NX;     // two rows from each neighbour
    unsigned hphase = 0u;                                 // bit k: parity of the next phase of hb[k]
    bool halo_failed = false;
    const float* hist_of_slot = nullptr;   // this slot's history, from the band's first row

    if (tid == 0) {
        for (int i = 0; i < 6; ++i) mbar_init(bars + i, 1);
        fence_mbar_init();
        s_fail = 0;
    }
    __syncthreads();
    // After a wait gives up, the CTA issues no further copies and waits no more
    // (the sweep's results are then invalid and the host reports the error); it
    // keeps meeting the cluster barriers so that no CTA is left behind, and thread 0
    // finally waits, again bounded, for the copies it issued that have not landed.
    auto wait_level = [&](int q) {
        if (failed) return;
        const unsigned par = (phase >> q) & 1u;
        if (!mbar_test_wait(bars + q, par) && (s_fail || !mbar_wait_bounded(bars + q, par))) {
            failed = true;
            s_fail = 1;
            return;
        }
        phase ^= 1u << q;
        pending &= ~(1u << q);
    };
    // M_m's halo rows, pushed by the neighbours in their step m-2 (bounded wait)
    auto wait_halo = [&](int k) {
        if (!halo_failed && !mbar_wait_bounded(hb + k, (hphase >> k) & 1u)) halo_failed = true;
        hphase ^= 1u << k;
    };
    auto issue_level = [&](int l) {    // thread 0 only
        if (failed || s_fail || l == a.skip_copy_level) return;
        const int q = l % 3;
        mbar_expect_tx(bars + q, band_bytes);
        tma_load_1d(U + q * band, hist_of_slot + (long long)l * g.NP, band_bytes, bars + q);
        pending |= 1u << q;
    };

    for (int slot = (int)cl_id(); slot < a.slots; slot += (int)cl_count()) {
        const ShotDesc sd = a.shots[slot];
        if (!sd.active) break;
        const float* al = a.alpha + (long long)sd.model * g.NP;
        const float kf = __ldg(a.kfac + sd.model);
        hist_of_slot = a.uhist + (long long)slot * a.u_slot_stride + (long long)b.z0 * g.pitch;
        // prefetch levels nt (u_{nt+1}) and nt-1 (u_nt) for the first reverse step
        if (tid == 0) {
            fence_proxy_async();
            for (int l = g.nt; l >= g.nt - 1 && l >= 0; --l) issue_level(l);
        }
        for (int i = tid; i < 3 * bufsz; i += blockDim.x) sm[i] = 0.0f;
        for (int i = tid; i < b.Rk * SP; i += blockDim.x) {
            const int r = i / SP, xx = i - r * SP;
            const int z = b.z0 + r;
            const int q = 2 * (i - xx % W) + xx % W;   // W columns of alpha, then W of 1-kappa
            AO[q] = xx < g.NX ? __ldg(al + (long long)z * g.pitch + xx) : 0.0f;
            AO[q + W] = xx < g.NX ? one_minus_kappa_of(kf, damp_at(z, xx, a.dampx, a.dampz, g)) : 0.0f;
        }
        // receivers in this thread's strip (at most two), as walk rows and columns of the thread
        int j0 = -1, c0 = 0, r0 = -1, j1 = -1, c1 = 0, r1 = -1;
        if (live)
            for (int i = 0; i < g.nrec; ++i) {
                const int rz = __ldg(a.rec_z + i) - b.z0 - st.r_begin;
                const int cx = __ldg(a.rec_x + i) - x;
                if (cx < 0 || cx >= W || rz < 0 || rz >= st.nrows) continue;
                const int j = up ? st.nrows - 1 - rz : rz;
                if (j0 < 0) { j0 = j; c0 = cx; r0 = i; }
                else if (j1 < 0) { j1 = j; c1 = cx; r1 = i; }
            }
        const bool warp_seed = __any_sync(0xffffffffu, j0 >= 0);
        const float* seed = a.seed + (long long)slot * g.nt * g.nrec + (long long)(g.nt - 1) * g.nrec;
        float s0 = j0 >= 0 ? __ldg(seed + r0) : 0.0f;
        float s1 = j1 >= 0 ? __ldg(seed + r1) : 0.0f;
        Vec<W> lam[RPT], mu[RPT], gv[RPT], gk[RPT];
#pragma unroll
        for (int j = 0; j < RPT; ++j) lam[j] = mu[j] = gv[j] = gk[j] = vsplat<W>(0.0f);
        // levels nt and nt-1 are read at the first step: thread 0 waits for them here;
        // every later level and halo is waited for by thread 0 at the end of the step
        // before the one that reads it, and the step's closing barrier publishes it
        if (tid == 0) {
            wait_level(g.nt % 3);
            if (g.nt >= 1) wait_level((g.nt - 1) % 3);
        }
        __syncthreads();
        cl_sync();

        // step t reads M_{t+3} = a lambda_{t+3} (buffer kc = t % 3) and writes
        // M_{t+2} (buffer kn = (t+2) % 3); as in the forward, only the halo rows
        // are waited for (three buffers).  The history ring uses the same
        // indices: u_{t+1} in kc, u_{t+2} in the third, level t-1 refills kn.
        // The time loop, specialised per thread variant (walk direction, full
        // strip, receivers in the warp) and chosen once per slot, so that the
        // loop-carried registers stay put.  Returns the buffer of M_2.
        auto time_loop = [&](auto full_c, auto seed_c, auto up_c) {
            constexpr bool F = decltype(full_c)::value, S = decltype(seed_c)::value, UPW = decltype(up_c)::value;
            int kc = (g.nt - 1) % 3, kn = (g.nt + 1) % 3;
            for (int t = g.nt - 1; t >= 0; --t) {
                const int k3 = 3 - kc - kn;
                const float* cb = M + kc * bufsz;
                float* nb = M + kn * bufsz;
                const HaloDst hd{smem_addr(nb), smem_addr(hb + kn)};
                // refill the buffer of level t+2 (last read at step t+1) with level t-1
                if (tid == 0) {
                    mbar_expect_tx(hb + kn, halo_bytes);
                    if (t >= 1) {
                        fence_proxy_async();
                        issue_level(t - 1);
                    }
                }
                if (live) {
                    adj_strip<RPT, W, SP, F, S, UPW>(cb, nb, hd, b, AO, U + kc * band, U + k3 * band, lam, mu, gv,
                                                     gk, st, x, xw, j0, c0, s0, j1, c1, s1);
                    finish_edges<SP, W>(nb, hd, b, st, x, ew);
                }
                // next step's seeds
                if (S && t >= 1) {
                    seed -= g.nrec;
                    if (j0 >= 0) s0 = __ldg(seed + r0);
                    if (j1 >= 0) s1 = __ldg(seed + r1);
                }
                // step t-1 reads M_{t+2} (buffer kn, its halo rows pushed by the neighbours
                // in their step t) and history level t-1 (ring slot kn, issued above)
                if (tid == 0 && t >= 1) {
                    wait_halo(kn);
                    wait_level(kn);
                }
                __syncthreads();
                kc = kn;   // (t-1) % 3 = (t+2) % 3
                kn = k3;   // (t+1) % 3
            }
            return kc;
        };
        using Yes = integral_c<true>;
        using No = integral_c<false>;
        int kc;
        if (up) {
            if (warp_seed) kc = full ? time_loop(Yes{}, Yes{}, Yes{}) : time_loop(No{}, Yes{}, Yes{});
            else kc = full ? time_loop(Yes{}, No{}, Yes{}) : time_loop(No{}, No{}, Yes{});
        } else {
            if (warp_seed) kc = full ? time_loop(Yes{}, Yes{}, No{}) : time_loop(No{}, Yes{}, No{});
            else kc = full ? time_loop(Yes{}, No{}, No{}) : time_loop(No{}, No{}, No{});
        }
        if (tid == 0) wait_halo(kc);   // M_2's halo rows (pushed at step 0, not read) have all landed
        if (live) {
            const int rw = up ? st.r_begin + st.nrows - 1 : st.r_begin;
            const int d = up ? -SP : SP;
            float* gvo = a.gv + (long long)slot * g.NP + (long long)(b.z0 + rw) * g.pitch + x;
            float* gko = a.gk + (long long)slot * g.NP + (long long)(b.z0 + rw) * g.pitch + x;
#pragma unroll
            for (int j = 0; j < RPT; ++j)
                if (j < st.nrows) {
                    st_cols<W>(gvo + j * d, gv[j]);
                    st_cols<W>(gko + j * d, gk[j]);
                }
        }
        __syncthreads();
    }
    if (tid == 0)
        for (int q = 0; q < 3; ++q)
            if ((pending >> q) & 1u && !mbar_wait_bounded(bars + q, (phase >> q) & 1u)) atomicOr(a.err, 2);
    if (failed) atomicOr(a.err, 1);
    if (halo_failed) atomicOr(a.err, 4);
}

}  // namespace
}  // namespace seis
