// noalloc.cu -- forward sweep that allocates no device memory.
//
// Some callers cannot call cudaMalloc once they are running: hosts whose
// allocator reserved the device's memory up front (frameworks that
// pre-allocate most of HBM for their own pool), latency-critical loops that
// may not take cudaMalloc's implicit device-wide synchronisation, and plugin
// hosts that forbid allocation inside their callbacks.  seis_forward_noalloc
// serves them: it computes the records of one model with the same kernels as
// seis_vel_to_seis, but its workspace is a fixed file-scope device array
// (kNoAllocScratchBytes, held by every GPU that loads the library until the
// process exits) instead of engine-owned allocations.
//
// The host-side name of a __device__ array is only a stand-in for the device
// address, so the array's device address is looked up once per device with
// cudaGetSymbolAddress (with that device current) and passed to the kernels.
// All calls share the array and it keeps the last call's contents; every
// buffer that must start at zero is cleared on each call.  Calls whose work
// overlaps on the GPU (different streams, or different host threads) race on
// the array and must be ordered by the caller.  The first call on a device
// performs the address look-up, so make it before any stream capture.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/seis_gb300.h"
#include "errors.h"
#include "prep_kernels.cuh"
#include "sweep_kernels.cuh"

using namespace seis;

namespace {

constexpr size_t kNoAllocScratchBytes = (size_t)8 << 20;   // SEIS_NOALLOC_SCRATCH_BYTES
static_assert(kNoAllocScratchBytes == SEIS_NOALLOC_SCRATCH_BYTES, "header and library disagree");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
void* g_scratch_ptr[kMaxDevices] = {};

int fail(int code, const char* msg)
{
    set_thread_error(msg);
    return code;
}

int fail_cuda(const char* what, cudaError_t e)
{
    set_thread_error(std::string("seis_forward_noalloc: ") + what + " failed: " + cudaGetErrorString(e));
    return SEIS_E_CUDA;
}

// Byte layout of the scratch array for one geometry; every region starts on 256 bytes.
struct Layout {
    size_t alpha, kfac, p, u, smod, rec, shots, dampx, dampz, ricker, src_z, src_x, rec_off, tstart, tlist, total;
};

size_t up256(size_t n) { return (n + 255) / 256 * 256; }

Layout layout_for(long long NP, int pitch, int NZ, int nt, int nshots, int nrec, int ntiles)
{
    Layout L{};
    size_t o = 0;
    auto take = [&](size_t bytes) { size_t at = o; o += up256(std::max<size_t>(bytes, 1)); return at; };
    L.alpha = take(sizeof(float) * NP);
    L.kfac = take(sizeof(float));
    L.p = take(sizeof(float) * 3 * NP);
    L.u = take(sizeof(float) * 2 * NP);
    L.smod = take(sizeof(float) * nt);
    L.rec = take(sizeof(float) * (size_t)nt * nrec);
    L.shots = take(sizeof(ShotDesc));
    L.dampx = take(sizeof(float) * pitch);
    L.dampz = take(sizeof(float) * NZ);
    L.ricker = take(sizeof(double) * nt);
    L.src_z = take(sizeof(int) * nshots);
    L.src_x = take(sizeof(int) * nshots);
    L.rec_off = take(sizeof(int) * nrec);
    L.tstart = take(sizeof(int) * (ntiles + 1));
    L.tlist = take(sizeof(int) * nrec);
    L.total = o;
    return L;
}

// Device address of the scratch array on the current device; looked up on the
// first call per device.
int scratch_address(unsigned char** out)
{
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(SEIS_E_CUDA, "seis_forward_noalloc: cudaGetDevice failed");
    if (dev < 0 || dev >= kMaxDevices) return fail(SEIS_E_INVALID, "seis_forward_noalloc: device index out of range");
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_ptr[dev]) {
        void* ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr) return fail_cuda("cudaGetSymbolAddress", e);
        g_scratch_ptr[dev] = ptr;
    }
    *out = (unsigned char*)g_scratch_ptr[dev];
    return 0;
}

int ricker_host(double freq, double dt, int nt, std::vector<double>& w)
{
    int nw = (int)(2.2 / freq / dt);
    nw = 2 * (nw / 2) + 1;
    const int nc = nw / 2 + 1;
    if (nt < nw) return -1;
    w.assign(nt, 0.0);
    for (int k = 1; k <= nw; ++k) {
        const double a = (double)(nc - k) * freq * dt * M_PI;
        const double b = a * a;
        w[k - 1] = (1.0 - 2.0 * b) * std::exp(-b);
    }
    return nw;
}

}  // namespace

extern "C" int seis_forward_noalloc(const SeisGeometry* G, const double* vec, double* result, void* stream)
{
    set_thread_error("");
    if (!G || !vec || !result) return fail(SEIS_E_INVALID, "seis_forward_noalloc: null geometry, vec or result");
    if (G->nz < 1 || G->nx < 1 || G->nbc < 2 || G->nt < 1 || !(G->dx > 0) || !(G->dt > 0) || !(G->freq > 0))
        return fail(SEIS_E_INVALID, "seis_forward_noalloc: invalid grid, spacing, step or frequency");
    if (G->nshots < 1 || !G->src_z || !G->src_x || G->nrec < 1 || !G->rec_z || !G->rec_x)
        return fail(SEIS_E_INVALID, "seis_forward_noalloc: need >= 1 shot and >= 1 receiver");
    const int NZ = G->nz + 2 * G->nbc, NX = G->nx + 2 * G->nbc;
    if ((long long)NZ * NX > (1LL << 28)) return fail(SEIS_E_INVALID, "seis_forward_noalloc: padded grid too large");
    for (int s = 0; s < G->nshots; ++s)
        if (G->src_z[s] < 0 || G->src_z[s] >= NZ || G->src_x[s] < 0 || G->src_x[s] >= NX)
            return fail(SEIS_E_INVALID, "seis_forward_noalloc: source outside the padded grid");
    for (int r = 0; r < G->nrec; ++r)
        if (G->rec_z[r] < 0 || G->rec_z[r] >= NZ || G->rec_x[r] < 0 || G->rec_x[r] >= NX)
            return fail(SEIS_E_INVALID, "seis_forward_noalloc: receiver outside the padded grid");
    std::vector<double> ricker;
    if (ricker_host(G->freq, G->dt, G->nt, ricker) < 0)
        return fail(SEIS_E_INVALID, "seis_forward_noalloc: nt is smaller than the Ricker wavelet");

    GridDev g{};
    const int pitch = (NX + 31) / 32 * 32;
    g.NZ = NZ; g.NX = NX; g.pitch = pitch;
    g.xlo = G->nbc; g.xhi = G->nbc + G->nx;
    g.NP = (long long)NZ * pitch;
    g.nt = G->nt; g.nrec = G->nrec;
    const int tiles_x = (NX + kTX - 1) / kTX, tiles_z = (NZ + kTZ - 1) / kTZ, ntiles = tiles_x * tiles_z;
    const Layout L = layout_for(g.NP, pitch, NZ, G->nt, G->nshots, G->nrec, ntiles);
    if (L.total > kNoAllocScratchBytes) {
        char msg[256];
        snprintf(msg, sizeof msg,
                 "seis_forward_noalloc: this geometry needs %zu bytes of scratch; the no-allocation path holds %zu "
                 "(padded grids up to about 400k points)", L.total, kNoAllocScratchBytes);
        return fail(SEIS_E_INVALID, msg);
    }

    unsigned char* base = nullptr;
    int rc = scratch_address(&base);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;

    // constants of the geometry (host-computed, copied from pageable memory)
    std::vector<float> dampx(pitch, 0.0f), dampz(NZ, 0.0f);
    {
        const double a = (G->nbc - 1) * G->dx;
        const double kappa = 3.0 * std::log(1e7) / (2.0 * a);
        for (int i = 0; i < G->nbc; ++i) {
            const double r = (i * G->dx) / a;
            const float d = (float)(kappa * (r * r));
            dampx[G->nbc - 1 - i] = d;
            dampx[G->nx + G->nbc + i] = d;
            dampz[G->nbc - 1 - i] = d;
            dampz[G->nz + G->nbc + i] = d;
        }
    }
    std::vector<int> rec_off(G->nrec), tstart(ntiles + 1, 0), tlist;
    {
        std::vector<std::vector<int>> per(ntiles);
        for (int r = 0; r < G->nrec; ++r) {
            rec_off[r] = G->rec_z[r] * pitch + G->rec_x[r];
            per[(G->rec_z[r] / kTZ) * tiles_x + G->rec_x[r] / kTX].push_back(r);
        }
        for (int t = 0; t < ntiles; ++t) {
            tstart[t] = (int)tlist.size();
            tlist.insert(tlist.end(), per[t].begin(), per[t].end());
        }
        tstart[ntiles] = (int)tlist.size();
    }
    auto cp = [&](size_t off, const void* src, size_t bytes) -> int {
        cudaError_t e = cudaMemcpyAsync(base + off, src, bytes, cudaMemcpyHostToDevice, st);
        return e == cudaSuccess ? 0 : fail_cuda("cudaMemcpyAsync", e);
    };
    if ((rc = cp(L.dampx, dampx.data(), sizeof(float) * pitch))) return rc;
    if ((rc = cp(L.dampz, dampz.data(), sizeof(float) * NZ))) return rc;
    if ((rc = cp(L.ricker, ricker.data(), sizeof(double) * G->nt))) return rc;
    if ((rc = cp(L.src_z, G->src_z, sizeof(int) * G->nshots))) return rc;
    if ((rc = cp(L.src_x, G->src_x, sizeof(int) * G->nshots))) return rc;
    if ((rc = cp(L.rec_off, rec_off.data(), sizeof(int) * G->nrec))) return rc;
    if ((rc = cp(L.tstart, tstart.data(), sizeof(int) * (ntiles + 1)))) return rc;
    if (!tlist.empty() && (rc = cp(L.tlist, tlist.data(), sizeof(int) * tlist.size()))) return rc;

    float* alpha = (float*)(base + L.alpha);
    float* kfac = (float*)(base + L.kfac);
    float* p = (float*)(base + L.p);
    float* u = (float*)(base + L.u);
    float* smod = (float*)(base + L.smod);
    float* rec = (float*)(base + L.rec);
    ShotDesc* shots = (ShotDesc*)(base + L.shots);
    ModelGeom mg{G->nz, G->nx, G->nbc, G->dt, G->dx};

    prep_models_kernel<<<std::max(1, (int)std::min<long long>((g.NP + 255) / 256, 152 * 16)), 256, 0, st>>>(
        g, mg, 1, vec, nullptr, alpha, kfac, nullptr, nullptr);

    FwdArgs a{};
    a.g = g;
    a.shots = shots;
    a.alpha = alpha;
    a.kfac = kfac;
    a.dampx = (const float*)(base + L.dampx);
    a.dampz = (const float*)(base + L.dampz);
    a.p = p;
    a.u = u;
    a.ulevels = 2;
    a.u_slot_stride = 2 * g.NP;
    a.smod = smod;
    a.rec = rec;
    a.tile_rec_start = (const int*)(base + L.tstart);
    a.tile_rec_list = (const int*)(base + L.tlist);
    a.rec_off = (const int*)(base + L.rec_off);
    const long long per_shot = (long long)G->nt * G->nrec;
    const dim3 grid(tiles_x, tiles_z, 1), block(kBX, kBZ);
    for (int s = 0; s < G->nshots; ++s) {
        chunk_setup_kernel<<<1, 128, 0, st>>>(g, mg, s, G->nshots, G->nshots, (const int*)(base + L.src_z),
                                              (const int*)(base + L.src_x), vec, nullptr,
                                              (const double*)(base + L.ricker), shots, smod, nullptr);
        cudaError_t e = cudaMemsetAsync(p, 0, sizeof(float) * 3 * g.NP, st);
        if (e == cudaSuccess) e = cudaMemsetAsync(u, 0, sizeof(float) * g.NP, st);
        if (e != cudaSuccess) return fail_cuda("cudaMemsetAsync", e);
        for (int t = 0; t < G->nt; ++t) fwd_step_kernel<false><<<grid, block, 0, st>>>(a, t);
        store_records_kernel<<<std::max(1, (int)std::min<long long>((per_shot + 255) / 256, 152 * 16)), 256, 0, st>>>(
            s, 1, per_shot, rec, result);
    }
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? 0 : fail_cuda("kernel launch", e);
}
