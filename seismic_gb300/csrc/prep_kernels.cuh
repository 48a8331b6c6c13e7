// prep_kernels.cuh -- per-call preparation and finalisation kernels of the
// FD engine: coefficient fields, per-shot source terms, record conversion,
// adjoint seeds, FP64 gradient accumulation, the edge-padding fold and the
// min_vel / misfit reductions.  Internal linkage (see sweep_kernels.cuh).
#pragma once
#include "common.cuh"

namespace seis {
namespace {

struct ModelGeom {
    int nz, nx, nbc;
    double dt, dx;
};

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// Velocity of padded point (z, x): edge padding of the model (cp.pad mode='edge').
__device__ __forceinline__ double padded_vel(const double* vec, int z, int x, const ModelGeom& mg)
{
    return vec[(size_t)clampi(z - mg.nbc, 0, mg.nz - 1) * mg.nx + clampi(x - mg.nbc, 0, mg.nx - 1)];
}

// prep_run / prep_run_diff: alpha = (v dt/dx)^2, alpha_d = 2 (dt/dx)^2 v dv.
__global__ void prep_models_kernel(GridDev g, ModelGeom mg, int nmodels, const double* __restrict__ vec,
                                   const double* __restrict__ vec_d, float* alpha, float* kfac,
                                   float* alpha_d, float* kdfac)
{
    const long long total = (long long)nmodels * g.NP;
    const size_t nv = (size_t)mg.nz * mg.nx + 1;
    const double dtdx = mg.dt / mg.dx;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < total;
         k += (long long)gridDim.x * blockDim.x) {
        const int m = (int)(k / g.NP);
        const long long i = k - (long long)m * g.NP;
        const int z = (int)(i / g.pitch), x = (int)(i - (long long)z * g.pitch);
        float a = 0.0f, ad = 0.0f;
        if (x < g.NX) {
            const double v = padded_vel(vec + nv * m, z, x, mg);
            const double r = v * dtdx;
            a = (float)(r * r);
            if (vec_d) ad = (float)(padded_vel(vec_d + nv * m, z, x, mg) * v * (2.0 * (dtdx * dtdx)));
        }
        alpha[k] = a;
        if (vec_d) alpha_d[k] = ad;
        if (i == 0) {
            kfac[m] = (float)(vec[nv * m + nv - 1] * mg.dt);
            if (vec_d) kdfac[m] = (float)(vec_d[nv * m + nv - 1] * mg.dt);
        }
    }
}

// Slot descriptors and source time functions of one chunk (one block per slot).
// s_mod = (v_src dt)^2 s  (core/seis_forward2.py:206-207);
// s_mod_diff = 2 v_src dv_src dt^2 s  (:253-254).
__global__ void chunk_setup_kernel(GridDev g, ModelGeom mg, int first_shot, int total_shots, int nshots,
                                   const int* __restrict__ src_z, const int* __restrict__ src_x,
                                   const double* __restrict__ vec, const double* __restrict__ vec_d,
                                   const double* __restrict__ ricker, ShotDesc* shots, float* smod,
                                   float* smod_d)
{
    const int slot = blockIdx.x;
    const int gs = first_shot + slot;
    const int active = gs < total_shots;
    const int m = active ? gs / nshots : 0;
    const int s = active ? gs % nshots : 0;
    const size_t nv = (size_t)mg.nz * mg.nx + 1;
    if (threadIdx.x == 0) {
        ShotDesc d;
        d.model = m;
        d.shot = s;
        d.src_off = src_z[s] * g.pitch + src_x[s];
        d.active = active;
        shots[slot] = d;
    }
    if (!active) return;
    const double v = padded_vel(vec + nv * m, src_z[s], src_x[s], mg);
    const double b = v * mg.dt;
    const double bdt = b * b;
    double bd = 0.0;
    if (vec_d) bd = 2.0 * (v * padded_vel(vec_d + nv * m, src_z[s], src_x[s], mg)) * (mg.dt * mg.dt);
    for (int t = threadIdx.x; t < g.nt; t += blockDim.x) {
        smod[(size_t)slot * g.nt + t] = (float)(bdt * ricker[t]);
        if (vec_d) smod_d[(size_t)slot * g.nt + t] = (float)(bd * ricker[t]);
    }
}

// FP32 records of a chunk -> caller's FP64 vector at the chunk's shot offset.
__global__ void store_records_kernel(int first_shot, int active_slots, long long per_shot,
                                     const float* __restrict__ rec, double* out)
{
    const long long total = (long long)active_slots * per_shot;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < total;
         k += (long long)gridDim.x * blockDim.x)
        out[(long long)first_shot * per_shot + k] = (double)rec[k];
}

// Adjoint seeds of a chunk: w, or F(vec) - w (core/seis_forward2.py:286-290).
__global__ void seeds_kernel(int first_shot, int active_slots, long long per_shot, int on_residual,
                             const double* __restrict__ result, const double* __restrict__ w, float* seed)
{
    const long long total = (long long)active_slots * per_shot;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < total;
         k += (long long)gridDim.x * blockDim.x) {
        const long long o = (long long)first_shot * per_shot + k;
        seed[k] = (float)(on_residual ? result[o] - w[o] : w[o]);
    }
}

// Add the chunk's per-slot FP32 sums into per-model FP64 accumulators, slots in
// order (deterministic for a given chunk size).  A model's consecutive slots are
// summed in registers (the same additions in the same order as adding each into
// memory), so a point's chain of slots does not wait on a memory round trip per slot.
__global__ void accumulate_kernel(GridDev g, const ShotDesc* __restrict__ shots, int slots,
                                  const float* __restrict__ gv, const float* __restrict__ gk, double* acc_v,
                                  double* acc_k)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < g.NP;
         i += (long long)gridDim.x * blockDim.x) {
        int cur = -1;
        double sv = 0.0, sk = 0.0;
        for (int s = 0; s < slots; ++s) {
            const ShotDesc d = shots[s];
            if (!d.active) break;
            if (d.model != cur) {
                if (cur >= 0) {
                    acc_v[(long long)cur * g.NP + i] = sv;
                    acc_k[(long long)cur * g.NP + i] = sk;
                }
                cur = d.model;
                sv = acc_v[(long long)cur * g.NP + i];
                sk = acc_k[(long long)cur * g.NP + i];
            }
            sv += (double)gv[(long long)s * g.NP + i];
            sk += (double)gk[(long long)s * g.NP + i];
        }
        if (cur >= 0) {
            acc_v[(long long)cur * g.NP + i] = sv;
            acc_k[(long long)cur * g.NP + i] = sk;
        }
    }
}

// dJ/dv on the model grid: (2/v) Gv summed over each cell's edge-padding
// preimage (unpad_edge_padded_gradient, core/seis_numerics.py:14-79).  The
// preimage of a cell is a rectangle (the edge cells own the whole padding
// strip beside them), so the sum is taken in two separable passes with short
// sequential chains (at most nbc+1 terms), in a fixed order:
//   fold_rows_kernel: rows[m][z][ix] = sum of Gv[m][z][x] over x in the column preimage of ix,
//   fold_cols_kernel: grad[m][iz][ix] = (2/v) sum of rows[m][z][ix] over z in the row preimage of iz.
__device__ __forceinline__ void fold_preimage(int i, int n, int nbc, int N, int& lo, int& hi)
{
    lo = i == 0 ? 0 : i + nbc;
    hi = i == n - 1 ? N : i + nbc + 1;
}
// Threads k < nmodels*NZ*ne take the edge columns (ix = 0 and nx-1: nbc+1 terms each),
// the others the interior (one term), so that no warp mixes a long chain with short ones.
__global__ void fold_rows_kernel(GridDev g, ModelGeom mg, int nmodels, const double* __restrict__ acc_v,
                                 double* rows)
{
    const int ne = mg.nx > 1 ? 2 : 1;                       // edge columns per row
    const long long nrow = (long long)nmodels * g.NZ;
    const long long nedge = nrow * ne, ninner = nrow * (mg.nx - ne);
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < nedge + ninner;
         k += (long long)gridDim.x * blockDim.x) {
        long long r;
        int ix;
        if (k < nedge) {
            r = k / ne;
            ix = k - r * ne == 0 ? 0 : mg.nx - 1;
        } else {
            r = (k - nedge) / (mg.nx - ne);
            ix = 1 + (int)(k - nedge - r * (mg.nx - ne));
        }
        const int m = (int)(r / g.NZ), z = (int)(r - (long long)m * g.NZ);
        const int c = z * mg.nx + ix;
        int xlo, xhi;
        fold_preimage(ix, mg.nx, mg.nbc, g.NX, xlo, xhi);
        const double* av = acc_v + (long long)m * g.NP + (long long)z * g.pitch;
        double s = 0.0;
        for (int x = xlo; x < xhi; ++x) s += av[x];
        rows[(long long)m * g.NP + c] = s;
    }
}
__global__ void fold_cols_kernel(GridDev g, ModelGeom mg, int nmodels, const double* __restrict__ vec,
                                 const double* __restrict__ rows, double* grad)
{
    const size_t nv = (size_t)mg.nz * mg.nx + 1;
    const long long total = (long long)nmodels * mg.nz * mg.nx;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < total;
         k += (long long)gridDim.x * blockDim.x) {
        const int m = (int)(k / ((long long)mg.nz * mg.nx));
        const int c = (int)(k - (long long)m * mg.nz * mg.nx);
        const int iz = c / mg.nx, ix = c - iz * mg.nx;
        int zlo, zhi;
        fold_preimage(iz, mg.nz, mg.nbc, g.NZ, zlo, zhi);
        const double* rm = rows + (long long)m * g.NP + ix;
        double s = 0.0;
        for (int z = zlo; z < zhi; ++z) s += rm[(long long)z * mg.nx];
        grad[nv * m + c] = 2.0 / vec[nv * m + c] * s;
    }
}

// dJ/dmin_vel = -dt sum_x damp(x) Gk(x); one block per model, fixed-order tree.
__global__ void minvel_grad_kernel(GridDev g, ModelGeom mg, const double* __restrict__ dampx,
                                   const double* __restrict__ dampz, const double* __restrict__ acc_k,
                                   double* grad)
{
    __shared__ double red[1024];
    const int m = blockIdx.x;
    const double* ak = acc_k + (long long)m * g.NP;
    double s = 0.0;
    for (long long i = threadIdx.x; i < (long long)g.NZ * g.NX; i += blockDim.x) {
        const int z = (int)(i / g.NX), x = (int)(i - (long long)z * g.NX);
        const double d = (x < g.xlo || x >= g.xhi) ? dampx[x] : dampz[z];
        s += d * ak[(long long)z * g.pitch + x];
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if (threadIdx.x < st) red[threadIdx.x] += red[threadIdx.x + st];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const size_t nv = (size_t)mg.nz * mg.nx + 1;
        grad[nv * m + nv - 1] = -mg.dt * red[0];
    }
}

// misfit[m] = sum over the model's records of (result - w)^2 in a fixed order: partial
// sum t of kMisfitParts adds the records i = t (mod kMisfitParts) in increasing i, then a
// tree over the partial sums.  The partial sums of a model are spread over several blocks
// (misfit_partial_kernel, grid kMisfitParts/128 x models) and the tree takes one block per
// model (misfit_kernel).
constexpr int kMisfitParts = 1024;
__global__ void misfit_partial_kernel(long long per_model, const double* __restrict__ result,
                                      const double* __restrict__ w, double* part)
{
    const int m = blockIdx.y;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    double s = 0.0;
    for (long long i = t; i < per_model; i += kMisfitParts) {
        const double d = result[per_model * m + i] - w[per_model * m + i];
        s += d * d;
    }
    part[(long long)m * kMisfitParts + t] = s;
}
__global__ void __launch_bounds__(kMisfitParts) misfit_kernel(const double* __restrict__ part, double* misfit)
{
    __shared__ double red[kMisfitParts];
    const int m = blockIdx.x;
    red[threadIdx.x] = part[(long long)m * kMisfitParts + threadIdx.x];
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if (threadIdx.x < st) red[threadIdx.x] += red[threadIdx.x + st];
        __syncthreads();
    }
    if (threadIdx.x == 0) misfit[m] = red[0];
}

}  // namespace
}  // namespace seis
