// optim.cu -- FP64 device kernels of the optimiser and priors that call the engine.
//
// seis_lbfgs_direction: the L-BFGS two-loop recursion d = -H g, which the
// reference runs as two single-block CUDA kernels (lbfgs_backward /
// lbfgs_forward, jcottaar/seismic core/seis_numerics.py:450-565) between
// host-side steps of its optimiser (core/seis_numerics.py:372-392).  Here one
// block handles one problem, so many inversions' directions are computed in
// a single launch; inner products are FP64 block reductions.
//   backward: for i = m-1..0: al_i = ro_i <s_i, q>;  q -= al_i y_i     (q = -g)
//   scale:    r = h_diag q
//   forward:  for i = 0..m-1: b_i = ro_i <y_i, r>;  r += (al_i - b_i) s_i
// The reference's forward loop also visits i = m, whose stored row and ro, al
// entries are still zero, which changes nothing; this loop stops at m - 1.
#include <cuda_runtime.h>

#include <string>

#include "../../include/seis_gb300.h"
#include "errors.h"

namespace {

constexpr int kOptThreads = 512;

__device__ double block_sum(double v, double* red)
{
    red[threadIdx.x] = v;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    const double r = red[0];
    __syncthreads();
    return r;
}

// The two-loop recursion of one problem by one block (m stored pairs).
__device__ void two_loop(int n, int m, const double* __restrict__ Sp, const double* __restrict__ Yp,
                         const double* __restrict__ rop, double* __restrict__ alp, const double* __restrict__ gp,
                         double h, double* __restrict__ dp, double* red)
{
    for (int i = threadIdx.x; i < n; i += blockDim.x) dp[i] = -gp[i];
    __syncthreads();
    for (int k = m - 1; k >= 0; --k) {
        double part = 0.0;
        for (int i = threadIdx.x; i < n; i += blockDim.x) part += Sp[(size_t)k * n + i] * dp[i];
        const double a = rop[k] * block_sum(part, red);
        if (threadIdx.x == 0) alp[k] = a;
        for (int i = threadIdx.x; i < n; i += blockDim.x) dp[i] -= a * Yp[(size_t)k * n + i];
        __syncthreads();
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) dp[i] *= h;
    __syncthreads();
    for (int k = 0; k < m; ++k) {
        double part = 0.0;
        for (int i = threadIdx.x; i < n; i += blockDim.x) part += Yp[(size_t)k * n + i] * dp[i];
        const double b = rop[k] * block_sum(part, red);
        const double c = alp[k] - b;
        for (int i = threadIdx.x; i < n; i += blockDim.x) dp[i] += c * Sp[(size_t)k * n + i];
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kOptThreads) lbfgs_two_loop_kernel(
    int n, int mcap, const int* __restrict__ num_old, const double* __restrict__ S, const double* __restrict__ Y,
    const double* __restrict__ ro, double* __restrict__ al, const double* __restrict__ g,
    const double* __restrict__ h_diag, double* __restrict__ d)
{
    __shared__ double red[kOptThreads];
    const int p = blockIdx.x;
    const int m = min(max(num_old[p], 0), mcap);
    two_loop(n, m, S + (size_t)p * mcap * n, Y + (size_t)p * mcap * n, ro + (size_t)p * mcap, al + (size_t)p * mcap,
             g + (size_t)p * n, h_diag[p], d + (size_t)p * n, red);
}

// ---------------------------------------------------------------------------
// Deterministic FP64 reductions of one problem per block (fixed order, so every
// caller -- the host-driven optimiser and the device-resident one -- gets the same
// bits): 0 <a, b>, 1 sum |a|, 2 max |a|.
__device__ double block_max(double v, double* red)
{
    red[threadIdx.x] = v;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
        __syncthreads();
    }
    const double r = red[0];
    __syncthreads();
    return r;
}
__device__ double vec_dot(int n, const double* a, const double* b, double* red)
{
    double part = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) part = __dadd_rn(part, __dmul_rn(a[i], b[i]));
    return block_sum(part, red);
}
__device__ double vec_sumabs(int n, const double* a, double* red)
{
    double part = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) part = __dadd_rn(part, fabs(a[i]));
    return block_sum(part, red);
}
__device__ double vec_maxabs(int n, const double* a, double* red)
{
    double part = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) part = fmax(part, fabs(a[i]));
    return block_max(part, red);
}

__global__ void __launch_bounds__(kOptThreads) reduce_kernel(int n, int op, const double* __restrict__ a,
                                                             const double* __restrict__ b, double* out)
{
    __shared__ double red[kOptThreads];
    const int p = blockIdx.x;
    const double* ap = a + (size_t)p * n;
    const double r = op == 0 ? vec_dot(n, ap, b + (size_t)p * n, red)
                             : (op == 1 ? vec_sumabs(n, ap, red) : vec_maxabs(n, ap, red));
    if (threadIdx.x == 0) out[p] = r;
}

// ---------------------------------------------------------------------------
// Device-resident L-BFGS with a strong-Wolfe line search: the reference's bfgs and
// _strong_wolfe (core/seis_numerics.py:138-277, 307-448; torch's LBFGS with
// lswolfe.lua) as a state machine, one block per problem.  Each step consumes the
// objective and gradient at the point the problem asked for last and runs its
// control flow up to the next point to evaluate (or to the end), so an optimisation
// needs no host read per evaluation.  Every scalar expression keeps the reference's
// evaluation order and rounds each operation (no contracted multiply-adds); inner
// products, |.| sums and maxima are the reductions above, so a host-driven run with
// the same reductions gives the same bits.
enum : int { kPcX0 = 0, kPcLsFirst = 1, kPcBracket = 2, kPcZoom = 3, kPcDone = 4 };
constexpr int kMaxLs = 25;
constexpr double kC1 = 1e-4, kC2 = 0.9, kLsTolChange = 1e-9;

struct LbfgsHdr {
    int pc, n_iter, cur_index, current_evals, ls_iter, ls_func_evals;
    int low, high, insuf, ls_done, nb, max_iter;
    double tol_grad, tol_change;
    double loss, prev_loss, h_diag, t, f0, gtd, d_norm;
    double t_prev, f_prev, gtd_prev, f_new, gtd_new;
    double b[2], bf[2], bgtd[2];
};
constexpr size_t kHdrBytes = 256;
static_assert(sizeof(LbfgsHdr) <= kHdrBytes, "header");

__host__ __device__ size_t lbfgs_state_bytes(int n, int max_iter)
{
    const size_t m = (size_t)max_iter + 1;
    const size_t bytes = kHdrBytes + 8 * ((size_t)7 * n + 2 * m * n + 2 * m);
    return (bytes + 255) / 256 * 256;
}

// Python's max(a, b) / min(a, b) on floats: the first argument unless the second is
// strictly greater / smaller.
__device__ __forceinline__ double py_max(double a, double b) { return b > a ? b : a; }
__device__ __forceinline__ double py_min(double a, double b) { return b < a ? b : a; }

// _cubic_interpolate (core/seis_numerics.py:279-304)
__device__ double cubic_interpolate(double x1, double f1, double g1, double x2, double f2, double g2, bool bounded,
                                    double lo, double hi)
{
    double xmin_bound, xmax_bound;
    if (bounded) {
        xmin_bound = lo;
        xmax_bound = hi;
    } else if (x1 <= x2) {
        xmin_bound = x1;
        xmax_bound = x2;
    } else {
        xmin_bound = x2;
        xmax_bound = x1;
    }
    const double d1 = __dsub_rn(__dadd_rn(g1, g2), __ddiv_rn(__dmul_rn(3.0, __dsub_rn(f1, f2)), __dsub_rn(x1, x2)));
    const double d2_square = __dsub_rn(__dmul_rn(d1, d1), __dmul_rn(g1, g2));
    if (d2_square >= 0) {
        const double d2 = __dsqrt_rn(d2_square);
        double min_pos;
        if (x1 <= x2)
            min_pos = __dsub_rn(x2, __dmul_rn(__dsub_rn(x2, x1), __ddiv_rn(__dsub_rn(__dadd_rn(g2, d2), d1),
                                                                         __dadd_rn(__dsub_rn(g2, g1), __dmul_rn(2.0, d2)))));
        else
            min_pos = __dsub_rn(x1, __dmul_rn(__dsub_rn(x1, x2), __ddiv_rn(__dsub_rn(__dadd_rn(g1, d2), d1),
                                                                         __dadd_rn(__dsub_rn(g1, g2), __dmul_rn(2.0, d2)))));
        return py_min(py_max(min_pos, xmin_bound), xmax_bound);
    }
    return __ddiv_rn(__dadd_rn(xmin_bound, xmax_bound), 2.0);
}

__global__ void __launch_bounds__(kOptThreads) lbfgs_step_kernel(int n, int max_iter, size_t stride, char* state,
                                                                 const double* __restrict__ f_in,
                                                                 const double* __restrict__ g_in, double* x_eval,
                                                                 int* done_out, const double* __restrict__ x0,
                                                                 double tol_grad, double tol_change)
{
    __shared__ double red[kOptThreads];
    const int p = blockIdx.x;
    char* base = state + (size_t)p * stride;
    LbfgsHdr* gh = reinterpret_cast<LbfgsHdr*>(base);
    const int mcap = max_iter + 1;
    double* x = reinterpret_cast<double*>(base + kHdrBytes);
    double* d = x + n;
    double* fg = d + n;      // flat_grad
    double* pfg = fg + n;    // prev_flat_grad
    double* gp = pfg + n;    // g_prev of the line search
    double* bg[2] = {gp + n, gp + 2 * n};     // bracket_g
    double* S = gp + 3 * n;                   // old_stps [mcap][n]
    double* Y = S + (size_t)mcap * n;         // old_dirs [mcap][n]
    double* ro = Y + (size_t)mcap * n;
    double* al = ro + mcap;
    double* xe = x_eval + (size_t)p * n;
    const int tid = threadIdx.x, nth = blockDim.x;
    auto copy = [&](double* dst, const double* src) {
        for (int i = tid; i < n; i += nth) dst[i] = src[i];
        __syncthreads();
    };
    auto eval_at = [&](double t, const double* dd) {       // x_eval = x + t d
        for (int i = tid; i < n; i += nth) xe[i] = __dadd_rn(x[i], __dmul_rn(t, dd[i]));
        __syncthreads();
    };
    if (x0) {
        // initialisation: the first point to evaluate is x0
        if (tid == 0) {
            LbfgsHdr h{};
            h.pc = kPcX0;
            h.max_iter = max_iter;
            h.tol_grad = tol_grad;
            h.tol_change = tol_change;
            *gh = h;
            done_out[p] = 0;
        }
        const double* x0p = x0 + (size_t)p * n;
        for (int i = tid; i < n; i += nth) {
            x[i] = x0p[i];
            xe[i] = x0p[i];
        }
        return;
    }
    LbfgsHdr H = *gh;
    if (H.pc == kPcDone) return;
    const double fin = f_in[p];
    const double* gin = g_in + (size_t)p * n;
    const int max_eval = H.max_iter * 5 / 4;
    switch (H.pc) {
    case kPcX0: goto after_x0;
    case kPcLsFirst: goto after_ls_first;
    case kPcBracket: goto after_bracket_eval;
    default: goto after_zoom_eval;
    }

after_x0:
    H.loss = fin;
    copy(fg, gin);
    H.current_evals = 1;
    if (vec_maxabs(n, fg, red) <= H.tol_grad) goto finish;
    H.n_iter = 0;
    H.cur_index = 0;
    H.h_diag = 1.0;

iter_start:
    H.n_iter += 1;
    if (H.n_iter == 1) {
        for (int i = tid; i < n; i += nth) d[i] = -fg[i];
        __syncthreads();
        H.h_diag = 1.0;
    } else {
        // y = flat_grad - prev_flat_grad and s = d t into the next free history rows
        double* y = Y + (size_t)H.cur_index * n;
        double* s = S + (size_t)H.cur_index * n;
        for (int i = tid; i < n; i += nth) {
            y[i] = __dsub_rn(fg[i], pfg[i]);
            s[i] = __dmul_rn(d[i], H.t);
        }
        __syncthreads();
        const double ys = vec_dot(n, y, s, red);
        if (ys > 1e-10) {
            if (tid == 0) ro[H.cur_index] = __ddiv_rn(1.0, ys);
            H.cur_index += 1;
            H.h_diag = __ddiv_rn(ys, vec_dot(n, y, y, red));
        }
        __syncthreads();
        two_loop(n, H.cur_index, S, Y, ro, al, fg, H.h_diag, d, red);
        __syncthreads();
    }
    copy(pfg, fg);
    H.prev_loss = H.loss;
    if (H.n_iter == 1) H.t = py_min(1.0, __ddiv_rn(1.0, vec_sumabs(n, fg, red)));
    else H.t = 1.0;
    H.gtd = vec_dot(n, fg, d, red);
    // _strong_wolfe(x, t, d, f = loss, g = flat_grad, gtd)
    H.d_norm = vec_maxabs(n, d, red);
    H.f0 = H.loss;
    eval_at(H.t, d);
    H.pc = kPcLsFirst;
    goto out;

after_ls_first:
    H.f_new = fin;
    H.ls_func_evals = 1;
    H.gtd_new = vec_dot(n, gin, d, red);
    H.t_prev = 0.0;
    H.f_prev = H.f0;
    copy(gp, fg);
    H.gtd_prev = H.gtd;
    H.ls_done = 0;
    H.ls_iter = 0;
    goto bracket_loop;

after_bracket_eval:
    H.f_new = fin;
    H.ls_func_evals += 1;
    H.gtd_new = vec_dot(n, gin, d, red);
    H.ls_iter += 1;

bracket_loop:
    if (H.ls_iter < kMaxLs) {
        const double armijo = __dadd_rn(H.f0, __dmul_rn(__dmul_rn(kC1, H.t), H.gtd));
        if (H.f_new > armijo || (H.ls_iter > 1 && H.f_new >= H.f_prev)) goto bracket_two;
        if (fabs(H.gtd_new) <= __dmul_rn(-kC2, H.gtd)) {
            // the strong Wolfe conditions hold at t
            H.b[0] = H.t;
            H.bf[0] = H.f_new;
            copy(bg[0], gin);
            H.nb = 1;
            H.ls_done = 1;
            goto bracket_end;
        }
        if (H.gtd_new >= 0) goto bracket_two;
        const double min_step = __dadd_rn(H.t, __dmul_rn(0.01, __dsub_rn(H.t, H.t_prev)));
        const double max_step = __dmul_rn(H.t, 10.0);
        const double tmp = H.t;
        H.t = cubic_interpolate(H.t_prev, H.f_prev, H.gtd_prev, H.t, H.f_new, H.gtd_new, true, min_step, max_step);
        H.t_prev = tmp;
        H.f_prev = H.f_new;
        copy(gp, gin);
        H.gtd_prev = H.gtd_new;
        eval_at(H.t, d);
        H.pc = kPcBracket;
        goto out;
    }

    goto bracket_end;

bracket_two:
    // a bracket [t_prev, t]
    H.b[0] = H.t_prev;
    H.b[1] = H.t;
    H.bf[0] = H.f_prev;
    H.bf[1] = H.f_new;
    copy(bg[0], gp);
    copy(bg[1], gin);
    H.bgtd[0] = H.gtd_prev;
    H.bgtd[1] = H.gtd_new;
    H.nb = 2;

bracket_end:
    if (H.ls_iter == kMaxLs) {
        H.b[0] = 0.0;
        H.b[1] = H.t;
        H.bf[0] = H.f0;
        H.bf[1] = H.f_new;
        copy(bg[0], fg);
        copy(bg[1], gin);
        H.nb = 2;
    }
    H.insuf = 0;
    if (H.bf[0] <= H.bf[H.nb - 1]) {
        H.low = 0;
        H.high = 1;
    } else {
        H.low = 1;
        H.high = 0;
    }

zoom_loop:
    if (!H.ls_done && H.ls_iter < kMaxLs) {
        if (__dmul_rn(fabs(__dsub_rn(H.b[1], H.b[0])), H.d_norm) < kLsTolChange) goto ls_end;
        H.t = cubic_interpolate(H.b[0], H.bf[0], H.bgtd[0], H.b[1], H.bf[1], H.bgtd[1], false, 0.0, 0.0);
        const double bmax = py_max(H.b[0], H.b[1]), bmin = py_min(H.b[0], H.b[1]);
        const double eps = __dmul_rn(0.1, __dsub_rn(bmax, bmin));
        if (py_min(__dsub_rn(bmax, H.t), __dsub_rn(H.t, bmin)) < eps) {
            if (H.insuf || H.t >= bmax || H.t <= bmin) {
                if (fabs(__dsub_rn(H.t, bmax)) < fabs(__dsub_rn(H.t, bmin))) H.t = __dsub_rn(bmax, eps);
                else H.t = __dadd_rn(bmin, eps);
                H.insuf = 0;
            } else {
                H.insuf = 1;
            }
        } else {
            H.insuf = 0;
        }
        eval_at(H.t, d);
        H.pc = kPcZoom;
        goto out;
    }
    goto ls_end;

after_zoom_eval:
    H.f_new = fin;
    H.ls_func_evals += 1;
    H.gtd_new = vec_dot(n, gin, d, red);
    H.ls_iter += 1;
    {
        const double armijo = __dadd_rn(H.f0, __dmul_rn(__dmul_rn(kC1, H.t), H.gtd));
        const int lo = H.low, hi = H.high;
        if (H.f_new > armijo || H.f_new >= H.bf[lo]) {
            H.b[hi] = H.t;
            H.bf[hi] = H.f_new;
            copy(bg[hi], gin);
            H.bgtd[hi] = H.gtd_new;
            if (H.bf[0] <= H.bf[1]) {
                H.low = 0;
                H.high = 1;
            } else {
                H.low = 1;
                H.high = 0;
            }
        } else {
            if (fabs(H.gtd_new) <= __dmul_rn(-kC2, H.gtd)) {
                H.ls_done = 1;
            } else if (__dmul_rn(H.gtd_new, __dsub_rn(H.b[hi], H.b[lo])) >= 0) {
                H.b[hi] = H.b[lo];
                H.bf[hi] = H.bf[lo];
                copy(bg[hi], bg[lo]);
                H.bgtd[hi] = H.bgtd[lo];
            }
            H.b[lo] = H.t;
            H.bf[lo] = H.f_new;
            copy(bg[lo], gin);
            H.bgtd[lo] = H.gtd_new;
        }
    }
    goto zoom_loop;

ls_end:
    // the line search returns (bracket_f[low], bracket_g[low], bracket[low], evaluations)
    H.loss = H.bf[H.low];
    copy(fg, bg[H.low]);
    H.t = H.b[H.low];
    for (int i = tid; i < n; i += nth) x[i] = __dadd_rn(x[i], __dmul_rn(H.t, d[i]));
    __syncthreads();
    H.current_evals += H.ls_func_evals;
    if (H.n_iter == H.max_iter) goto finish;
    if (H.current_evals >= max_eval) goto finish;
    if (vec_maxabs(n, fg, red) <= H.tol_grad) goto finish;
    {
        double part = 0.0;
        for (int i = tid; i < n; i += nth) part = fmax(part, fabs(__dmul_rn(d[i], H.t)));
        if (block_max(part, red) <= H.tol_change) goto finish;
    }
    if (fabs(__dsub_rn(H.loss, H.prev_loss)) < H.tol_change) goto finish;
    goto iter_start;

finish:
    copy(xe, x);
    H.pc = kPcDone;
    if (tid == 0) done_out[p] = 1;

out:
    __syncthreads();
    if (tid == 0) *gh = H;
}

// Smoothed total-variation prior (core/seis_prior.py:112-176), fused cost +
// gradient for m models at once, one block per model:
//   cost = lam * mean over all vertical and horizontal neighbour differences d of
//          sqrt(d^2 + eps^2);  grad = lam * d cost / d x  (0 for min_vel).
// Each block sums in a fixed order, so a model's result does not depend on m.
__global__ void __launch_bounds__(kOptThreads) tv_prior_kernel(int nz, int nx, double eps2, double lam,
                                                               const double* __restrict__ X, double* cost,
                                                               double* grad)
{
    __shared__ double red[kOptThreads];
    const int mi = blockIdx.x;
    const size_t nv = (size_t)nz * nx + 1;
    const double* m = X + nv * mi;
    double* g = grad + nv * mi;
    const double n = (double)(nz - 1) * nx + (double)nz * (nx - 1);
    double part = 0.0;
    for (int c = threadIdx.x; c < nz * nx; c += blockDim.x) {
        const int z = c / nx, x = c - z * nx;
        const double v = m[c];
        double gc = 0.0;
        if (z + 1 < nz) {          // vertical difference d1(z, x) = m[z+1, x] - m[z, x]
            const double d = m[c + nx] - v;
            const double sq = sqrt(d * d + eps2);
            part += sq;
            gc -= d / sq;
        }
        if (z > 0) {
            const double d = v - m[c - nx];
            gc += d / sqrt(d * d + eps2);
        }
        if (x + 1 < nx) {          // horizontal difference d2(z, x) = m[z, x+1] - m[z, x]
            const double d = m[c + 1] - v;
            const double sq = sqrt(d * d + eps2);
            part += sq;
            gc -= d / sq;
        }
        if (x > 0) {
            const double d = v - m[c - 1];
            gc += d / sqrt(d * d + eps2);
        }
        g[c] = lam * gc / n;
    }
    const double total = block_sum(part, red);
    if (threadIdx.x == 0) {
        cost[mi] = lam * total / n;
        g[nv - 1] = 0.0;
    }
}

}  // namespace

extern "C" int seis_tv_prior(int32_t m, int32_t nz, int32_t nx, double epsilon, double lam, const double* x,
                             double* cost, double* grad, void* stream)
{
    if (m < 1 || nz < 1 || nx < 1 || (nz < 2 && nx < 2) || !x || !cost || !grad) {
        seis::set_thread_error("seis_tv_prior: invalid sizes or null pointer");
        return SEIS_E_INVALID;
    }
    tv_prior_kernel<<<m, kOptThreads, 0, (cudaStream_t)stream>>>(nz, nx, epsilon * epsilon, lam, x, cost, grad);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        seis::set_thread_error(std::string("seis_tv_prior: launch failed: ") + cudaGetErrorString(e));
        return SEIS_E_CUDA;
    }
    return 0;
}

extern "C" int seis_reduce(int32_t nprob, int32_t n, int32_t op, const double* a, const double* b, double* out,
                           void* stream)
{
    if (nprob < 1 || n < 1 || op < 0 || op > 2 || !a || !out || (op == 0 && !b)) {
        seis::set_thread_error("seis_reduce: invalid sizes, operation or null pointer");
        return SEIS_E_INVALID;
    }
    reduce_kernel<<<nprob, kOptThreads, 0, (cudaStream_t)stream>>>(n, op, a, b, out);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        seis::set_thread_error(std::string("seis_reduce: launch failed: ") + cudaGetErrorString(e));
        return SEIS_E_CUDA;
    }
    return 0;
}

extern "C" int64_t seis_lbfgs_state_bytes(int32_t n, int32_t max_iter)
{
    if (n < 1 || max_iter < 1) return 0;
    return (int64_t)lbfgs_state_bytes(n, max_iter);
}

extern "C" int seis_lbfgs_step(int32_t nprob, int32_t n, int32_t max_iter, double tolerance_grad,
                               double tolerance_change, const double* x0, const double* f, const double* g,
                               void* state, double* x_eval, int32_t* done, void* stream)
{
    if (nprob < 1 || n < 1 || max_iter < 1 || !state || !x_eval || !done || (!x0 && (!f || !g))) {
        seis::set_thread_error("seis_lbfgs_step: invalid sizes or null pointer");
        return SEIS_E_INVALID;
    }
    if (reinterpret_cast<uintptr_t>(state) % 256) {
        seis::set_thread_error("seis_lbfgs_step: state must be 256-byte aligned");
        return SEIS_E_INVALID;
    }
    lbfgs_step_kernel<<<nprob, kOptThreads, 0, (cudaStream_t)stream>>>(
        n, max_iter, lbfgs_state_bytes(n, max_iter), static_cast<char*>(state), f, g, x_eval, done, x0, tolerance_grad,
        tolerance_change);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        seis::set_thread_error(std::string("seis_lbfgs_step: launch failed: ") + cudaGetErrorString(e));
        return SEIS_E_CUDA;
    }
    return 0;
}

extern "C" int seis_lbfgs_direction(int32_t nprob, int32_t n, int32_t m_cap, const int32_t* num_old,
                                    const double* old_stps, const double* old_dirs, const double* ro, double* al,
                                    const double* grad, const double* h_diag, double* d, void* stream)
{
    if (nprob < 1 || n < 1 || m_cap < 1 || !num_old || !old_stps || !old_dirs || !ro || !al || !grad || !h_diag || !d) {
        seis::set_thread_error("seis_lbfgs_direction: invalid sizes or null pointer");
        return SEIS_E_INVALID;
    }
    lbfgs_two_loop_kernel<<<nprob, kOptThreads, 0, (cudaStream_t)stream>>>(n, m_cap, num_old, old_stps, old_dirs, ro,
                                                                          al, grad, h_diag, d);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        seis::set_thread_error(std::string("seis_lbfgs_direction: launch failed: ") + cudaGetErrorString(e));
        return SEIS_E_CUDA;
    }
    return 0;
}
