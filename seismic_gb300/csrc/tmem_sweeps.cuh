// tmem_sweeps.cuh -- cluster-resident sweeps that keep per-point state which no
// neighbour reads in tensor memory (sm_103a): the adjoint and the forward.
//
// The adjoint of cluster_kernels.cuh keeps lambda, mu and the two gradient sums of
// its points in registers and alpha, 1-kappa and a three-level history ring in
// shared memory.  That footprint (about 11 KB per band row) needs 16-CTA
// clusters, and only seven of them fit on the GPU (112 SMs).  This variant moves
// what only the owning thread touches out of the register file and shared memory
// into the SM's tensor memory (TMEM, 128 lanes x 512 columns of 32 bits, unused by
// a stencil): alpha, the gradient sums Gv and Gk, and the history level u_{t+2}
// that the previous step read (carried instead of re-read).  1 - kappa is rebuilt
// from the separable sponge profile in registers, and the history ring shrinks to
// two levels.  A band row then takes about 6.4 KB of shared memory, so a 10-CTA
// cluster holds a shot (32-row bands, 13 resident clusters, 130 SMs), and each
// point moves about 22 bytes through shared memory per step instead of 35.
//
// Tensor memory: warp w of the CTA may address lanes 32 (w % 4) .. 32 (w % 4) + 31,
// so thread l of warp w owns lane 32 (w % 4) + l; the warps sharing a lane quarter
// take 8 RPT columns each (in the order w / 4), 8 per walk row of the thread's strip:
//   [alpha(x), alpha(x+1), u(x), u(x+1), Gv(x), Gv(x+1), Gk(x), Gk(x+1)].
// Warp 0 allocates 512 columns at entry and frees them at exit (also after a
// timed-out wait).  Only one CTA of a kernel with this much shared memory fits on
// an SM, so the allocation never waits for another CTA's columns.
// tcgen05.ld / st / wait are warp-collective (.sync.aligned): every thread of a
// strip group with rows executes them, including the lanes past the grid's last
// column, whose shared stores, halo pushes and outputs are masked off, and a
// __syncwarp() reconverges the warp before each of them that follows lane-dependent
// code.
//
// The arithmetic is adj_strip's, in the same order, so the gradients are bitwise
// those of the other adjoint sweeps.
#pragma once
#include "cluster_kernels.cuh"

namespace seis {
namespace {

// ---------------------------------------------------------------------------
// tcgen05 helpers
// ---------------------------------------------------------------------------
constexpr unsigned kTmemCols = 512;

__device__ __forceinline__ void tmem_alloc(unsigned* slot, unsigned ncols = kTmemCols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(unsigned taddr, unsigned ncols = kTmemCols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tmem_fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tmem_fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// 8 consecutive columns of this thread's lane; the values are valid after tmem_wait_ld(v).
__device__ __forceinline__ void tmem_ld8(unsigned taddr, float (&v)[8])
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7])
                 : "r"(taddr)
                 : "memory");
}
// Wait for this thread's tensor-memory loads; the operands tie the loaded registers
// to the wait so that no use is scheduled before it.
__device__ __forceinline__ void tmem_wait_ld(float (&v)[8])
{
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+f"(v[0]), "+f"(v[1]), "+f"(v[2]), "+f"(v[3]), "+f"(v[4]), "+f"(v[5]), "+f"(v[6]), "+f"(v[7])
                 :
                 : "memory");
}
__device__ __forceinline__ void tmem_ld2(unsigned taddr, float (&v)[2])
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x2.b32 {%0, %1}, [%2];" : "=f"(v[0]), "=f"(v[1]) : "r"(taddr) : "memory");
}
__device__ __forceinline__ void tmem_wait_ld(float (&v)[2])
{
    asm volatile("tcgen05.wait::ld.sync.aligned;" : "+f"(v[0]), "+f"(v[1]) : : "memory");
}
__device__ __forceinline__ void tmem_ld4(unsigned taddr, float (&v)[4])
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3])
                 : "r"(taddr)
                 : "memory");
}
__device__ __forceinline__ void tmem_wait_ld(float (&v)[4])
{
    asm volatile("tcgen05.wait::ld.sync.aligned;" : "+f"(v[0]), "+f"(v[1]), "+f"(v[2]), "+f"(v[3]) : : "memory");
}
__device__ __forceinline__ void tmem_st2(unsigned taddr, float2 a)
{
    asm volatile("tcgen05.st.sync.aligned.32x32b.x2.b32 [%0], {%1, %2};" ::"r"(taddr), "f"(a.x), "f"(a.y) : "memory");
}
__device__ __forceinline__ void tmem_st4(unsigned taddr, float2 a, float2 b)
{
    asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1, %2, %3, %4};" ::"r"(taddr), "f"(a.x), "f"(a.y),
                 "f"(b.x), "f"(b.y)
                 : "memory");
}
__device__ __forceinline__ void tmem_st8(unsigned taddr, float2 a, float2 b, float2 c, float2 d)
{
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"r"(taddr),
                 "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y), "f"(d.x), "f"(d.y)
                 : "memory");
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// Columns of one walk row in a thread's tensor-memory block.
constexpr unsigned kTmAlpha = 0, kTmU = 2, kTmG = 4, kTmRow = 8;

// ---------------------------------------------------------------------------
// strip of the adjoint step, column pairs, per-point state in tensor memory
//   mu = (1-k) mu + Lap(a lambda') [+ seed],  lambda = lambda' + mu,
//   Gv += lambda (u_{t+2} - (1-k) u_{t+1}),  Gk += lambda u_{t+1},  M' = a lambda;
// u_{t+1} is read from the shared ring (U1) and carried in tensor memory as the next
// step's u_{t+2}.  1 - kappa: the band's row profile OMR in shared memory (one value
// per row, a broadcast load) or, in the side bands, the thread's column values.
// `live`: the thread's columns lie on the grid (else only the warp-collective
// tensor-memory accesses run for it).
struct OmCols {
    float col[2];     // 1 - kappa of columns x, x+1 where they lie in a side band
    unsigned side;    // bit w: column x + w lies in a side band
};
// ---------------------------------------------------------------------------
template <int RPT, int SP, bool FULL, bool SEED, bool UP>
__device__ __forceinline__ void adj_strip_tm(const float* __restrict__ cb, float* __restrict__ nb, const HaloDst& hd,
                                             const Band<SP>& b, const float* __restrict__ U1, unsigned trow,
                                             const float* __restrict__ OMR, const OmCols& om, float2 (&lam)[RPT],
                                             float2 (&mu)[RPT],
                                             const Strip& s, int x, const XWrap<2>& xw, bool live, int j0, int c0,
                                             float s0, int j1, int c1, float s1)
{
    const int r0 = UP ? s.r_begin + s.nrows - 1 : s.r_begin;
    constexpr int D = UP ? -1 : 1;
    const float* col = cb + (r0 + 2) * SP + x + 2;
    float2 w0 = ld_cols<2>(col - 2 * D * SP), w1 = ld_cols<2>(col - D * SP), w2 = ld_cols<2>(col),
           w3 = ld_cols<2>(col + D * SP);
    const int o0 = r0 * SP + x;
    float* out = nb + (r0 + 2) * SP + x + 2;
#pragma unroll
    for (int j = 0; j < RPT; ++j) {
        if (FULL || j < s.nrows) {
            const unsigned tr = trow + kTmRow * (unsigned)j;
            float tv[8];
            // lanes may have diverged only at the strip's start and after a halo push (rows 0, 1)
            if (j <= 2) __syncwarp();
            tmem_ld8(tr, tv);
            const float2 w4 = ld_cols<2>(col + (j + 2) * D * SP);
            float2 h1, h2;
            horiz_sums<2>(col + j * D * SP, xw, w2, h1, h2);
            const float2 u1 = ld_cols<2>(U1 + o0 + j * D * SP);
            const float2 t1 = vadd(h1, vadd(w3, w1)), t2 = vadd(h2, vadd(w4, w0));
            const float orow = OMR[r0 + j * D];
            const float2 omv = make_float2((om.side & 1u) ? om.col[0] : orow, (om.side & 2u) ? om.col[1] : orow);
            float2 m = vfma(omv, mu[j], stencil_lap(w2, t1, t2));
            if (SEED) {
                // the receivers' seeds by selects (no lane-dependent branch before the wait)
                m.x = j == j0 && c0 == 0 ? m.x + s0 : m.x;
                m.y = j == j0 && c0 == 1 ? m.y + s0 : m.y;
                m.x = j == j1 && c1 == 0 ? m.x + s1 : m.x;
                m.y = j == j1 && c1 == 1 ? m.y + s1 : m.y;
                __syncwarp();
            }
            const float2 lv = vadd(lam[j], m);
            mu[j] = m;
            lam[j] = lv;
            tmem_wait_ld(tv);
            const float2 av = make_float2(tv[kTmAlpha], tv[kTmAlpha + 1]);
            const float2 u2 = make_float2(tv[kTmU], tv[kTmU + 1]);
            float2 gv = make_float2(tv[kTmG], tv[kTmG + 1]), gk = make_float2(tv[kTmG + 2], tv[kTmG + 3]);
            gv = vfma(lv, vfma(vneg(omv), u1, u2), gv);
            gk = vfma(lv, u1, gk);
            tmem_st8(tr, av, u1, gv, gk);      // alpha rewritten unchanged: one store per row
            const float2 mv = vmul(av, lv);
            // lanes past the grid's last column store into columns that are never read (the
            // row's tail and the next row's two leading columns, inside the same buffer)
            st_cols<2>(out + j * D * SP, mv);
            if (j < 2 && live) {
                if (!UP && s.push_top) push_up_cols<SP, 2>(hd, b, s.r_begin + j, x, mv);
                if (UP && s.push_bottom) push_down_cols<SP, 2>(hd, b, r0 - j, x, mv);
            }
            w0 = w1; w1 = w2; w2 = w3; w3 = w4;
        }
    }
}

// ---------------------------------------------------------------------------
// adjoint sweep (t = nt-1 .. 0), C-CTA clusters, column pairs
// smem: M[3][R+4][SP] (a*lambda) | U[2][R][SP] (history ring) | mbar[2] (history) |
//       mbar[3] (halos) | fail flag (8 B) | tensor-memory address (8 B) | OMR[R] (1 - kappa per band row)
// ---------------------------------------------------------------------------
template <int C, int RPT, int SP, int NTHR>
__global__ void __launch_bounds__(NTHR, 1) adj_cluster_tm_kernel(ClusterArgs a)
{
    static_assert(kTmRow * RPT * ((NTHR / 32 + 3) / 4) <= kTmemCols, "tensor-memory blocks exceed the allocation");
    constexpr int W = 2;
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
    float* U = sm + 3 * bufsz;                             // 2 history levels of the band
    uint64_t* bars = (uint64_t*)(U + 2 * band);            // band*4 is a multiple of 128 bytes
    uint64_t* hb = bars + 2;                               // halo mbarrier of each M buffer
    volatile int& s_fail = *(volatile int*)(bars + 5);
    unsigned* s_tmem = (unsigned*)(bars + 6);
    float* OMR = (float*)(bars + 7);
    const int tid = threadIdx.x;
    const int x = W * (tid % GW), gg = tid / GW;
    const Strip st = make_strip<SP>(b, gg, a.G, RPT);
    const bool up = gg == a.G - 1 && a.G > 1;
    const bool active = st.nrows > 0;                      // uniform over the strip group (its warps)
    const bool live = active && x < g.NX;
    const bool full = st.nrows == RPT;
    const unsigned band_bytes = (unsigned)(b.Rk * SP * 4);
    unsigned phase = 0u;    // bit i: parity of the next phase to wait for on history barrier i
    unsigned pending = 0u;  // (thread 0) bit i: a copy on barrier i whose completion it has not seen
    bool failed = false;
    const unsigned ew = live ? edge_work<SP, W>(b, st, x) : 0u;
    const XWrap<W> xw = make_xwrap<W>(x, g.NX);
    const unsigned halo_bytes = 16u * (unsigned)g.NX;     // two rows from each neighbour
    unsigned hphase = 0u;
    bool halo_failed = false;
    const float* hist_of_slot = nullptr;

    if (tid < 32) tmem_alloc(s_tmem);                      // warp 0
    if (tid == 0) {
        for (int i = 0; i < 5; ++i) mbar_init(bars + i, 1);
        fence_mbar_init();
        s_fail = 0;
    }
    tmem_fence_before_sync();
    __syncthreads();
    tmem_fence_after_sync();
    const unsigned warp = (unsigned)tid >> 5;
    // this thread's block: its warp's lane quarter, 64 columns per warp of the quarter
    const unsigned tbase = *s_tmem + ((32u * (warp & 3u)) << 16) + kTmRow * RPT * (warp >> 2);

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
    auto wait_halo = [&](int k) {
        if (!halo_failed && !mbar_wait_bounded(hb + k, (hphase >> k) & 1u)) halo_failed = true;
        hphase ^= 1u << k;
    };
    auto issue_level = [&](int l) {    // thread 0 only: level l into ring slot l % 2
        if (failed || s_fail || l == a.skip_copy_level) return;
        const int q = l & 1;
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
        if (tid == 0) {
            fence_proxy_async();
            issue_level(g.nt);          // u_{nt+1}: the first step's carried level
            if (g.nt >= 1) issue_level(g.nt - 1);
        }
        for (int i = tid; i < 3 * bufsz; i += blockDim.x) sm[i] = 0.0f;
        // 1 - kappa (separable sponge profile: band rows in shared memory, side-band columns in
        // registers) and, per walk row, alpha into tensor memory
        const int rw = up ? st.r_begin + st.nrows - 1 : st.r_begin;
        for (int r = tid; r < b.Rk; r += blockDim.x) OMR[r] = one_minus_kappa_of(kf, __ldg(a.dampz + b.z0 + r));
        OmCols omr;
        omr.side = 0u;
#pragma unroll
        for (int w = 0; w < W; ++w) {
            const int xc = x + w;
            const bool side = xc < g.xlo || xc >= g.xhi;
            omr.side |= (unsigned)side << w;
            omr.col[w] = live && side ? one_minus_kappa_of(kf, __ldg(a.dampx + xc)) : 0.0f;
        }
        if (active) {
#pragma unroll
            for (int j = 0; j < RPT; ++j) {
                const int z = b.z0 + (up ? rw - j : rw + j);
                const bool in = live && j < st.nrows;
                const float2 av = in ? __ldg(reinterpret_cast<const float2*>(al + (long long)z * g.pitch + x))
                                     : make_float2(0.0f, 0.0f);
                const unsigned tr = tbase + kTmRow * (unsigned)j;
                __syncwarp();
                tmem_st2(tr + kTmAlpha, av);
                tmem_st4(tr + kTmG, make_float2(0.0f, 0.0f), make_float2(0.0f, 0.0f));
            }
        }
        // receivers in this thread's strip (at most two)
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
        float2 lam[RPT], mu[RPT];
#pragma unroll
        for (int j = 0; j < RPT; ++j) lam[j] = mu[j] = make_float2(0.0f, 0.0f);
        // the first step's u_{t+2} (level nt) into the carried column, then its ring slot is free
        if (tid == 0) wait_level(g.nt & 1);
        __syncthreads();
        if (active) {
            const float* Un = U + (g.nt & 1) * band;
#pragma unroll
            for (int j = 0; j < RPT; ++j) {
                const float2 u = j < st.nrows ? ld_cols<2>(Un + (up ? rw - j : rw + j) * SP + x) : make_float2(0.0f, 0.0f);
                tmem_st2(tbase + kTmRow * (unsigned)j + kTmU, u);
            }
            tmem_wait_st();
        }
        if (tid == 0 && g.nt >= 1) wait_level((g.nt - 1) & 1);
        __syncthreads();
        cl_sync();

        // step t reads M_{t+3} (buffer t % 3) and writes M_{t+2} (buffer (t+2) % 3), history
        // level t (u_{t+1}) from ring slot t % 2; at its start thread 0 refills the other
        // slot (level t+1, read at step t+1 and now carried) with level t-1
        auto time_loop = [&](auto full_c, auto seed_c, auto up_c) {
            constexpr bool F = decltype(full_c)::value, S = decltype(seed_c)::value, UPW = decltype(up_c)::value;
            int kc = (g.nt - 1) % 3, kn = (g.nt + 1) % 3;
            for (int t = g.nt - 1; t >= 0; --t) {
                const int k3 = 3 - kc - kn;
                const float* cb = M + kc * bufsz;
                float* nb = M + kn * bufsz;
                const HaloDst hd{smem_addr(nb), smem_addr(hb + kn)};
                if (tid == 0) {
                    mbar_expect_tx(hb + kn, halo_bytes);
                    if (t >= 1) {
                        fence_proxy_async();
                        issue_level(t - 1);
                    }
                }
                if (active) {
                    adj_strip_tm<RPT, SP, F, S, UPW>(cb, nb, hd, b, U + (t & 1) * band, tbase, OMR, omr, lam, mu, st,
                                                     x, xw, live, j0, c0, s0, j1, c1, s1);
                    if (live) finish_edges<SP, W>(nb, hd, b, st, x, ew);
                    __syncwarp();
                    tmem_wait_st();
                }
                if (S && t >= 1) {
                    seed -= g.nrec;
                    if (j0 >= 0) s0 = __ldg(seed + r0);
                    if (j1 >= 0) s1 = __ldg(seed + r1);
                }
                if (tid == 0 && t >= 1) {
                    wait_halo(kn);
                    wait_level((t - 1) & 1);
                }
                __syncthreads();
                kc = kn;
                kn = k3;
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
        if (active) {
            const int d = up ? -SP : SP;
            float* gvo = a.gv + (long long)slot * g.NP + (long long)(b.z0 + rw) * g.pitch + x;
            float* gko = a.gk + (long long)slot * g.NP + (long long)(b.z0 + rw) * g.pitch + x;
#pragma unroll
            for (int j = 0; j < RPT; ++j)
                if (j < st.nrows) {
                    float tv[8];
                    __syncwarp();
                    tmem_ld8(tbase + kTmRow * (unsigned)j, tv);
                    tmem_wait_ld(tv);
                    if (live) {
                        st_cols<2>(gvo + j * d, make_float2(tv[kTmG], tv[kTmG + 1]));
                        st_cols<2>(gko + j * d, make_float2(tv[kTmG + 2], tv[kTmG + 3]));
                    }
                }
        }
        __syncthreads();
    }
    if (tid == 0)
        for (int q = 0; q < 2; ++q)
            if ((pending >> q) & 1u && !mbar_wait_bounded(bars + q, (phase >> q) & 1u)) atomicOr(a.err, 2);
    if (failed) atomicOr(a.err, 1);
    if (halo_failed) atomicOr(a.err, 4);
    tmem_fence_before_sync();
    __syncthreads();
    tmem_fence_after_sync();
    if (tid < 32) tmem_dealloc(*s_tmem);
}

}  // namespace
}  // namespace seis

namespace seis {
namespace {

// ---------------------------------------------------------------------------
// forward sweep with alpha in tensor memory (column pairs, no tangent)
//
// fwd_cluster_kernel with its band's alpha moved from shared memory into tensor
// memory: 2 columns per walk row of a thread (16 per warp at 8 rows; 128 columns
// allocated), read once per row and step with tcgen05.ld x2.  Each point then moves
// about 18 bytes through shared memory per step instead of 22.  Everything else --
// bands, strips, pushes, waits, history, records -- is fwd_cluster_kernel's, so the
// records and history are bitwise the same.
// ---------------------------------------------------------------------------
constexpr unsigned kFwdTmemCols = 128;

template <int RPT, int SP, bool FULL, bool SRC, bool UP>
__device__ __forceinline__ void fwd_strip_tm(const float* __restrict__ cb, float* __restrict__ nb, const HaloDst& hd,
                                             const Band<SP>& b, unsigned trow, const OneMinusKappa<RPT, 2>& om,
                                             float2 (&u)[RPT], const Strip& s, int x, const XWrap<2>& xw, bool live,
                                             int jsrc, int scol, float src)
{
    const int r0 = UP ? s.r_begin + s.nrows - 1 : s.r_begin;
    constexpr int D = UP ? -1 : 1;
    const float* col = cb + (r0 + 2) * SP + x + 2;
    float2 w0 = ld_cols<2>(col - 2 * D * SP), w1 = ld_cols<2>(col - D * SP), w2 = ld_cols<2>(col),
           w3 = ld_cols<2>(col + D * SP);
    float* out = nb + (r0 + 2) * SP + x + 2;
#pragma unroll
    for (int j = 0; j < RPT; ++j) {
        if (FULL || j < s.nrows) {
            float ta[2];
            if (j <= 2) __syncwarp();      // lanes diverge only at the strip's start and after a halo push
            tmem_ld2(trow + 2u * (unsigned)j, ta);
            const float2 w4 = ld_cols<2>(col + (j + 2) * D * SP);
            float2 h1, h2;
            horiz_sums<2>(col + j * D * SP, xw, w2, h1, h2);
            const float2 t1 = vadd(h1, vadd(w3, w1)), t2 = vadd(h2, vadd(w4, w0));
            const float2 lap = stencil_lap(w2, t1, t2);
            const float2 omu = vmul(om.at(j), u[j]);
            tmem_wait_ld(ta);
            float2 un = vfma(make_float2(ta[0], ta[1]), lap, omu);
            if (SRC) {                     // the source by selects: no lane-dependent branch
                un.x = j == jsrc && scol == 0 ? un.x + src : un.x;
                un.y = j == jsrc && scol == 1 ? un.y + src : un.y;
                __syncwarp();
            }
            u[j] = un;
            const float2 pn = vadd(w2, un);
            // lanes past the grid's last column store into never-read columns (see adj_strip_tm)
            st_cols<2>(out + j * D * SP, pn);
            if (j < 2 && live) {
                if (!UP && s.push_top) push_up_cols<SP, 2>(hd, b, s.r_begin + j, x, pn);
                if (UP && s.push_bottom) push_down_cols<SP, 2>(hd, b, r0 - j, x, pn);
            }
            w0 = w1; w1 = w2; w2 = w3; w3 = w4;
        }
    }
}

// smem: P[3][R+4][SP] | halo mbar[3] | S[nt] | receivers of the band (3 x nrec ints) | count |
//       tensor-memory address (4 B)
template <int C, int RPT, int SP, int NTHR>
__global__ void __launch_bounds__(NTHR, 1) fwd_cluster_tm_kernel(ClusterArgs a)
{
    constexpr int W = 2;
    constexpr int GW = SP / W;
    static_assert(2 * RPT * ((NTHR / 32 + 3) / 4) <= (int)kFwdTmemCols, "tensor-memory blocks exceed the allocation");
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
    float* P = sm;                                   // 3 buffers: p_m in buffer m % 3
    uint64_t* hb = (uint64_t*)(P + 3 * bufsz);       // halo mbarrier of each buffer
    float* SRC = (float*)(hb + 3);
    int* RL = (int*)(SRC + g.nt);                    // [3][nrec]: band row, column, receiver id
    int* nrl = RL + 3 * g.nrec;
    unsigned* s_tmem = (unsigned*)(nrl + 1);
    const int tid = threadIdx.x;
    const int x = W * (tid % GW), gg = tid / GW;
    const Strip st = make_strip<SP>(b, gg, a.G, RPT);
    const bool up = gg == a.G - 1 && a.G > 1;
    const bool active = st.nrows > 0;               // uniform over the strip group
    const bool live = active && x < g.NX;
    const bool full = st.nrows == RPT;
    const unsigned ew = live ? edge_work<SP, W>(b, st, x) : 0u;
    const XWrap<W> xw = make_xwrap<W>(x, g.NX);
    const unsigned halo_bytes = 16u * (unsigned)g.NX;
    unsigned hphase = 0u;
    bool halo_failed = false;
    const bool reads_halo = tid == 0 || st.r_begin < 2 || st.r_begin + st.nrows + 2 > b.Rk;
    if (tid < 32) tmem_alloc(s_tmem, kFwdTmemCols);
    if (tid == 0) {
        for (int k = 0; k < 3; ++k) mbar_init(hb + k, 1);
        fence_mbar_init();
    }
    tmem_fence_before_sync();
    __syncthreads();
    tmem_fence_after_sync();
    const unsigned warp = (unsigned)tid >> 5;
    const unsigned tbase = *s_tmem + ((32u * (warp & 3u)) << 16) + 2u * RPT * (warp >> 2);
    auto wait_halo = [&](int k) {
        if (!halo_failed && !mbar_wait_bounded(hb + k, (hphase >> k) & 1u)) halo_failed = true;
        hphase ^= 1u << k;
    };

    for (int slot = (int)cl_id(); slot < a.slots; slot += (int)cl_count()) {
        const ShotDesc sd = a.shots[slot];
        if (!sd.active) break;
        const float* al = a.alpha + (long long)sd.model * g.NP;
        const float kf = __ldg(a.kfac + sd.model);
        if (tid == 0) *nrl = 0;
        for (int i = tid; i < 3 * bufsz; i += blockDim.x) sm[i] = 0.0f;
        // 1 - kappa of the strip in registers, alpha of its walk rows in tensor memory
        OneMinusKappa<RPT, W> omr;
        {
            const int r0 = up ? st.r_begin + st.nrows - 1 : st.r_begin;
            omr.side = 0u;
#pragma unroll
            for (int w = 0; w < W; ++w) {
                const int xc = x + w;
                const bool side = xc < g.xlo || xc >= g.xhi;
                omr.side |= (unsigned)side << w;
                omr.col[w] = live && side ? one_minus_kappa_of(kf, __ldg(a.dampx + xc)) : 0.0f;
            }
#pragma unroll
            for (int j = 0; j < RPT; ++j) {
                const int z = b.z0 + (up ? r0 - j : r0 + j);
                const bool in = live && j < st.nrows;
                omr.row[j] = in ? one_minus_kappa_of(kf, __ldg(a.dampz + z)) : 0.0f;
                const float2 av = in ? __ldg(reinterpret_cast<const float2*>(al + (long long)z * g.pitch + x))
                                     : make_float2(0.0f, 0.0f);
                if (active) {
                    __syncwarp();
                    tmem_st2(tbase + 2u * (unsigned)j, av);
                }
            }
            if (active) {
                __syncwarp();
                tmem_wait_st();
            }
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
        int jsrc = -1;
        const int scol = sx - x;
        if (live && scol >= 0 && scol < W && sz >= st.r_begin && sz < st.r_begin + st.nrows)
            jsrc = up ? st.r_begin + st.nrows - 1 - sz : sz - st.r_begin;
        const bool warp_src = __any_sync(0xffffffffu, jsrc >= 0);
        float* rec = a.rec + (long long)slot * g.nt * g.nrec;
        float* hist = a.write_hist ? a.uhist + (long long)slot * a.u_slot_stride + (long long)b.z0 * g.pitch + x
                                   : nullptr;
        float2 u[RPT];
#pragma unroll
        for (int j = 0; j < RPT; ++j) u[j] = make_float2(0.0f, 0.0f);
        __syncthreads();
        const int nr = *nrl;
        const int gather0 = a.G > 2 ? (int)blockDim.x / a.G : 0;
        cl_sync();

        auto time_loop = [&](auto full_c, auto src_c, auto up_c) {
            constexpr bool F = decltype(full_c)::value, S = decltype(src_c)::value, U = decltype(up_c)::value;
            const long long hrow = (long long)(U ? st.r_begin + st.nrows - 1 : st.r_begin) * SP;
            int kc = 1;
            for (int t = 0; t < g.nt; ++t) {
                const int kn = kc == 2 ? 0 : kc + 1;
                const float* cb = P + kc * bufsz;
                float* nb = P + kn * bufsz;
                const HaloDst hd{smem_addr(nb), smem_addr(hb + kn)};
                if (tid == 0) mbar_expect_tx(hb + kn, halo_bytes);
                if (t > 0) {
                    if (reads_halo) wait_halo(kc);
                    for (int i = tid - gather0; i >= 0 && i < nr; i += blockDim.x) {
                        const int bo = Band<SP>::at(RL[i], RL[g.nrec + i]);
                        const long long ro = (long long)(t - 1) * g.nrec + RL[2 * g.nrec + i];
                        rec[ro] = cb[bo];
                    }
                }
                if (active) {
                    fwd_strip_tm<RPT, SP, F, S, U>(cb, nb, hd, b, tbase, omr, u, st, x, xw, live, jsrc, scol, SRC[t]);
                    if (live) {
                        finish_edges<SP, W>(nb, hd, b, st, x, ew);
                        if (hist) store_hist<RPT, W, SP, F, U>(hist + (long long)(t + 1) * g.NP + hrow, u, st.nrows);
                    }
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
        if (reads_halo) wait_halo(kc);
        const float* fb = P + kc * bufsz;
        for (int i = tid; i < nr; i += blockDim.x) {
            const int bo = Band<SP>::at(RL[i], RL[g.nrec + i]);
            const long long ro = (long long)(g.nt - 1) * g.nrec + RL[2 * g.nrec + i];
            rec[ro] = fb[bo];
        }
        cl_sync();
    }
    if (halo_failed) atomicOr(a.err, 4);
    tmem_fence_before_sync();
    __syncthreads();
    tmem_fence_after_sync();
    if (tid < 32) tmem_dealloc(*s_tmem, kFwdTmemCols);
}

}  // namespace
}  // namespace seis

namespace seis {
namespace {

// ---------------------------------------------------------------------------
// forward + tangent sweep with alpha and dalpha in tensor memory (column pairs)
//
// fwd_cluster_kernel<…, TAN> (16-CTA clusters, six wavefield buffers) with the band's
// alpha and dalpha in tensor memory (4 columns per walk row of a thread: alpha(x),
// alpha(x+1), dalpha(x), dalpha(x+1); one tcgen05.ld x4 per row and step) and the row
// profiles of 1 - kappa and -dkappa in shared memory (one broadcast load each per
// row), so that a thread's registers hold only u and du of its points: the register
// version spills at the 96-register cap.  The arithmetic is tan_strip's (the tangent
// increment lane by lane), so records and tangent records are bitwise the same.
// ---------------------------------------------------------------------------
template <int RPT, int SP, bool FULL, bool SRC, bool UP>
__device__ __forceinline__ void tan_strip_tm(const float* __restrict__ cb, float* __restrict__ nb,
                                             const float* __restrict__ dcb, float* __restrict__ dnb, const HaloDst& hd,
                                             const HaloDst& hdd, const Band<SP>& b, unsigned trow,
                                             const float* __restrict__ OMR, const float* __restrict__ NKR,
                                             const OmCols& om, const OmCols& nk, float2 (&u)[RPT], float2 (&du)[RPT],
                                             const Strip& s, int x, const XWrap<2>& xw, bool live, int jsrc, int scol,
                                             float src, float src_d)
{
    const int r0 = UP ? s.r_begin + s.nrows - 1 : s.r_begin;
    constexpr int D = UP ? -1 : 1;
    const int c0 = (r0 + 2) * SP + x + 2;
    const float* col = cb + c0;
    const float* dcol = dcb + c0;
    float2 w0 = ld_cols<2>(col - 2 * D * SP), w1 = ld_cols<2>(col - D * SP), w2 = ld_cols<2>(col),
           w3 = ld_cols<2>(col + D * SP);
    float2 v0 = ld_cols<2>(dcol - 2 * D * SP), v1 = ld_cols<2>(dcol - D * SP), v2 = ld_cols<2>(dcol),
           v3 = ld_cols<2>(dcol + D * SP);
#pragma unroll
    for (int j = 0; j < RPT; ++j) {
        if (FULL || j < s.nrows) {
            float ta[4];
            if (j <= 2) __syncwarp();      // lanes diverge only at the strip's start and after a halo push
            tmem_ld4(trow + 4u * (unsigned)j, ta);
            const float2 w4 = ld_cols<2>(col + (j + 2) * D * SP);
            const float2 v4 = ld_cols<2>(dcol + (j + 2) * D * SP);
            float2 h1, h2, g1, g2;
            horiz_sums<2>(col + j * D * SP, xw, w2, h1, h2);
            horiz_sums<2>(dcol + j * D * SP, xw, v2, g1, g2);
            const float2 t1 = vadd(h1, vadd(w3, w1)), t2 = vadd(h2, vadd(w4, w0));
            const float2 d1 = vadd(g1, vadd(v3, v1)), d2 = vadd(g2, vadd(v4, v0));
            const float2 L = stencil_lap(w2, t1, t2);
            const float2 dL = stencil_lap(v2, d1, d2);
            const float orow = OMR[r0 + j * D], nrow = NKR[r0 + j * D];
            const float2 omw = make_float2((om.side & 1u) ? om.col[0] : orow, (om.side & 2u) ? om.col[1] : orow);
            const float2 nkw = make_float2((nk.side & 1u) ? nk.col[0] : nrow, (nk.side & 2u) ? nk.col[1] : nrow);
            tmem_wait_ld(ta);
            const float2 av = make_float2(ta[0], ta[1]), adv = make_float2(ta[2], ta[3]);
            float2 un = fwd_increment(omw, u[j], av, L);
            float2 dun;
            dun.x = tan_increment_nkd(omw.x, du[j].x, av.x, dL.x, adv.x, L.x, nkw.x, u[j].x);
            dun.y = tan_increment_nkd(omw.y, du[j].y, av.y, dL.y, adv.y, L.y, nkw.y, u[j].y);
            if (SRC) {                     // the source by selects: no lane-dependent branch
                un.x = j == jsrc && scol == 0 ? un.x + src : un.x;
                un.y = j == jsrc && scol == 1 ? un.y + src : un.y;
                dun.x = j == jsrc && scol == 0 ? dun.x + src_d : dun.x;
                dun.y = j == jsrc && scol == 1 ? dun.y + src_d : dun.y;
                __syncwarp();
            }
            u[j] = un;
            du[j] = dun;
            const float2 pn = vadd(w2, un), dpn = vadd(v2, dun);
            // lanes past the grid's last column store into never-read columns (see adj_strip_tm)
            st_cols<2>(nb + c0 + j * D * SP, pn);
            st_cols<2>(dnb + c0 + j * D * SP, dpn);
            if (j < 2 && live) {
                if (!UP && s.push_top) {
                    push_up_cols<SP, 2>(hd, b, s.r_begin + j, x, pn);
                    push_up_cols<SP, 2>(hdd, b, s.r_begin + j, x, dpn);
                }
                if (UP && s.push_bottom) {
                    push_down_cols<SP, 2>(hd, b, r0 - j, x, pn);
                    push_down_cols<SP, 2>(hdd, b, r0 - j, x, dpn);
                }
            }
            w0 = w1; w1 = w2; w2 = w3; w3 = w4;
            v0 = v1; v1 = v2; v2 = v3; v3 = v4;
        }
    }
}

// smem: P[3][R+4][SP] | DP[3][R+4][SP] | halo mbar[3] | S[nt] | SD[nt] | OMR[R] | NKR[R] |
//       receivers of the band (3 x nrec ints) | count | tensor-memory address
template <int C, int RPT, int SP, int NTHR>
__global__ void __launch_bounds__(NTHR, 1) tan_cluster_tm_kernel(ClusterArgs a)
{
    constexpr int W = 2;
    constexpr int GW = SP / W;
    static_assert(4 * RPT * ((NTHR / 32 + 3) / 4) <= (int)kFwdTmemCols, "tensor-memory blocks exceed the allocation");
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
    float* P = sm;
    float* DP = P + 3 * bufsz;
    uint64_t* hb = (uint64_t*)(DP + 3 * bufsz);
    float* SRC = (float*)(hb + 3);
    float* SRCD = SRC + g.nt;
    float* OMR = SRCD + g.nt;
    float* NKR = OMR + R;
    int* RL = (int*)(NKR + R);
    int* nrl = RL + 3 * g.nrec;
    unsigned* s_tmem = (unsigned*)(nrl + 1);
    const int tid = threadIdx.x;
    const int x = W * (tid % GW), gg = tid / GW;
    const Strip st = make_strip<SP>(b, gg, a.G, RPT);
    const bool up = gg == a.G - 1 && a.G > 1;
    const bool active = st.nrows > 0;
    const bool live = active && x < g.NX;
    const bool full = st.nrows == RPT;
    const unsigned ew = live ? edge_work<SP, W>(b, st, x) : 0u;
    const XWrap<W> xw = make_xwrap<W>(x, g.NX);
    const unsigned halo_bytes = 32u * (unsigned)g.NX;   // two rows of each field from each neighbour
    unsigned hphase = 0u;
    bool halo_failed = false;
    const bool reads_halo = tid == 0 || st.r_begin < 2 || st.r_begin + st.nrows + 2 > b.Rk;
    if (tid < 32) tmem_alloc(s_tmem, kFwdTmemCols);
    if (tid == 0) {
        for (int k = 0; k < 3; ++k) mbar_init(hb + k, 1);
        fence_mbar_init();
    }
    tmem_fence_before_sync();
    __syncthreads();
    tmem_fence_after_sync();
    const unsigned warp = (unsigned)tid >> 5;
    const unsigned tbase = *s_tmem + ((32u * (warp & 3u)) << 16) + 4u * RPT * (warp >> 2);
    auto wait_halo = [&](int k) {
        if (!halo_failed && !mbar_wait_bounded(hb + k, (hphase >> k) & 1u)) halo_failed = true;
        hphase ^= 1u << k;
    };

    for (int slot = (int)cl_id(); slot < a.slots; slot += (int)cl_count()) {
        const ShotDesc sd = a.shots[slot];
        if (!sd.active) break;
        const float* al = a.alpha + (long long)sd.model * g.NP;
        const float* ald = a.alpha_d + (long long)sd.model * g.NP;
        const float kf = __ldg(a.kfac + sd.model);
        const float kdf = __ldg(a.kdfac + sd.model);
        if (tid == 0) *nrl = 0;
        for (int i = tid; i < 6 * bufsz; i += blockDim.x) sm[i] = 0.0f;
        for (int r = tid; r < b.Rk; r += blockDim.x) {
            const float dz = __ldg(a.dampz + b.z0 + r);
            OMR[r] = one_minus_kappa_of(kf, dz);
            NKR[r] = -__fmul_rn(kdf, dz);
        }
        OmCols omc, nkc;
        omc.side = 0u;
#pragma unroll
        for (int w = 0; w < W; ++w) {
            const int xc = x + w;
            const bool side = xc < g.xlo || xc >= g.xhi;
            omc.side |= (unsigned)side << w;
            omc.col[w] = live && side ? one_minus_kappa_of(kf, __ldg(a.dampx + xc)) : 0.0f;
            nkc.col[w] = live && side ? -__fmul_rn(kdf, __ldg(a.dampx + xc)) : 0.0f;
        }
        nkc.side = omc.side;
        if (active) {
            const int r0 = up ? st.r_begin + st.nrows - 1 : st.r_begin;
#pragma unroll
            for (int j = 0; j < RPT; ++j) {
                const int z = b.z0 + (up ? r0 - j : r0 + j);
                const bool in = live && j < st.nrows;
                const float2 av = in ? __ldg(reinterpret_cast<const float2*>(al + (long long)z * g.pitch + x))
                                     : make_float2(0.0f, 0.0f);
                const float2 adv = in ? __ldg(reinterpret_cast<const float2*>(ald + (long long)z * g.pitch + x))
                                      : make_float2(0.0f, 0.0f);
                __syncwarp();
                tmem_st4(tbase + 4u * (unsigned)j, av, adv);
            }
            __syncwarp();
            tmem_wait_st();
        }
        const float* smod = a.smod + (long long)slot * g.nt;
        const float* smd = a.smod_d + (long long)slot * g.nt;
        for (int i = tid; i < g.nt; i += blockDim.x) {
            SRC[i] = __ldg(smod + i);
            SRCD[i] = __ldg(smd + i);
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
        const int sz = sd.src_off / g.pitch - b.z0, sx = sd.src_off % g.pitch;
        int jsrc = -1;
        const int scol = sx - x;
        if (live && scol >= 0 && scol < W && sz >= st.r_begin && sz < st.r_begin + st.nrows)
            jsrc = up ? st.r_begin + st.nrows - 1 - sz : sz - st.r_begin;
        const bool warp_src = __any_sync(0xffffffffu, jsrc >= 0);
        float* rec = a.rec + (long long)slot * g.nt * g.nrec;
        float* drec = a.drec + (long long)slot * g.nt * g.nrec;
        float* hist = a.write_hist ? a.uhist + (long long)slot * a.u_slot_stride + (long long)b.z0 * g.pitch + x
                                   : nullptr;
        float2 u[RPT], du[RPT];
#pragma unroll
        for (int j = 0; j < RPT; ++j) u[j] = du[j] = make_float2(0.0f, 0.0f);
        __syncthreads();
        const int nr = *nrl;
        const int gather0 = a.G > 2 ? (int)blockDim.x / a.G : 0;
        cl_sync();

        auto time_loop = [&](auto full_c, auto src_c, auto up_c) {
            constexpr bool F = decltype(full_c)::value, S = decltype(src_c)::value, U = decltype(up_c)::value;
            const long long hrow = (long long)(U ? st.r_begin + st.nrows - 1 : st.r_begin) * SP;
            int kc = 1;
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
                    for (int i = tid - gather0; i >= 0 && i < nr; i += blockDim.x) {
                        const int bo = Band<SP>::at(RL[i], RL[g.nrec + i]);
                        const long long ro = (long long)(t - 1) * g.nrec + RL[2 * g.nrec + i];
                        rec[ro] = cb[bo];
                        drec[ro] = dcb[bo];
                    }
                }
                if (active) {
                    tan_strip_tm<RPT, SP, F, S, U>(cb, nb, dcb, dnb, hd, hdd, b, tbase, OMR, NKR, omc, nkc, u, du, st, x,
                                                   xw, live, jsrc, scol, SRC[t], SRCD[t]);
                    if (live) {
                        finish_edges<SP, W>(dnb, hdd, b, st, x, ew);
                        finish_edges<SP, W>(nb, hd, b, st, x, ew);
                        if (hist) store_hist<RPT, W, SP, F, U>(hist + (long long)(t + 1) * g.NP + hrow, u, st.nrows);
                    }
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
        if (reads_halo) wait_halo(kc);
        const float* fb = P + kc * bufsz;
        for (int i = tid; i < nr; i += blockDim.x) {
            const int bo = Band<SP>::at(RL[i], RL[g.nrec + i]);
            const long long ro = (long long)(g.nt - 1) * g.nrec + RL[2 * g.nrec + i];
            rec[ro] = fb[bo];
            drec[ro] = DP[kc * bufsz + bo];
        }
        cl_sync();
    }
    if (halo_failed) atomicOr(a.err, 4);
    tmem_fence_before_sync();
    __syncthreads();
    tmem_fence_after_sync();
    if (tid < 32) tmem_dealloc(*s_tmem, kFwdTmemCols);
}

}  // namespace
}  // namespace seis
