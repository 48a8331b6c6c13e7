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

__global__ void __launch_bounds__(kOptThreads) lbfgs_two_loop_kernel(
    int n, int mcap, const int* __restrict__ num_old, const double* __restrict__ S, const double* __restrict__ Y,
    const double* __restrict__ ro, double* __restrict__ al, const double* __restrict__ g,
    const double* __restrict__ h_diag, double* __restrict__ d)
{
    __shared__ double red[kOptThreads];
    const int p = blockIdx.x;
    const int m = min(max(num_old[p], 0), mcap);
    const double* Sp = S + (size_t)p * mcap * n;
    const double* Yp = Y + (size_t)p * mcap * n;
    const double* rop = ro + (size_t)p * mcap;
    double* alp = al + (size_t)p * mcap;
    const double* gp = g + (size_t)p * n;
    double* dp = d + (size_t)p * n;
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
    const double h = h_diag[p];
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
