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
//
// The geometry's constants (sponge profile, wavelet, source and receiver
// positions) travel by value as the parameters of one set-up kernel that
// writes them into the array: no host staging buffer is involved, so nothing
// of a call refers to host memory once the call has returned.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/seis_gb300.h"
#include "errors.h"
#include "host_setup.h"
#include "prep_kernels.cuh"
#include "sweep_kernels.cuh"

using namespace seis;

namespace seis {
namespace noalloc_detail {

// Limits of the by-value constants (SEIS_NOALLOC_MAX_*); the parameter block stays
// well inside the 32 KB kernel-parameter space.
constexpr int kMaxShots = SEIS_NOALLOC_MAX_SHOTS;
constexpr int kMaxRec = SEIS_NOALLOC_MAX_RECEIVERS;
constexpr int kMaxNbc = SEIS_NOALLOC_MAX_NBC;
constexpr int kMaxWavelet = SEIS_NOALLOC_MAX_WAVELET;

struct Consts {
    int nshots, nrec, nbc, nw, nz, nx, tiles_x, ntiles;
    float d1[kMaxNbc];             // sponge profile d1[i] (FP32, as the sweeps read it)
    double wavelet[kMaxWavelet];   // the Ricker wavelet's first nw samples (the rest are zero)
    int src_z[kMaxShots], src_x[kMaxShots];
    int rec_z[kMaxRec], rec_x[kMaxRec];
};
static_assert(sizeof(Consts) < 30000, "kernel parameter block too large");

// The geometry's constants into the scratch regions (one block; tile lists by thread 0,
// receivers of a tile in increasing order, as the engine builds them).
__global__ void noalloc_setup_kernel(Consts c, GridDev g, float* dampx, float* dampz, double* ricker, int* src_z,
                                     int* src_x, int* rec_off, int* tstart, int* tlist)
{
    for (int x = threadIdx.x; x < g.pitch; x += blockDim.x)
        dampx[x] = x < c.nbc ? c.d1[c.nbc - 1 - x]
                             : (x >= c.nx + c.nbc && x < c.nx + 2 * c.nbc ? c.d1[x - c.nx - c.nbc] : 0.0f);
    for (int z = threadIdx.x; z < g.NZ; z += blockDim.x)
        dampz[z] = z < c.nbc ? c.d1[c.nbc - 1 - z]
                             : (z >= c.nz + c.nbc && z < c.nz + 2 * c.nbc ? c.d1[z - c.nz - c.nbc] : 0.0f);
    for (int t = threadIdx.x; t < g.nt; t += blockDim.x) ricker[t] = t < c.nw ? c.wavelet[t] : 0.0;
    for (int s = threadIdx.x; s < c.nshots; s += blockDim.x) {
        src_z[s] = c.src_z[s];
        src_x[s] = c.src_x[s];
    }
    for (int r = threadIdx.x; r < c.nrec; r += blockDim.x) rec_off[r] = c.rec_z[r] * g.pitch + c.rec_x[r];
    if (threadIdx.x == 0) {
        int n = 0;
        for (int t = 0; t < c.ntiles; ++t) {
            tstart[t] = n;
            for (int r = 0; r < c.nrec; ++r)
                if ((c.rec_z[r] / kTZ) * c.tiles_x + c.rec_x[r] / kTX == t) tlist[n++] = r;
        }
        tstart[c.ntiles] = n;
    }
}

}  // namespace noalloc_detail
}  // namespace seis

using namespace seis::noalloc_detail;

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
int scratch_address(int dev, unsigned char** out)
{
    if (dev < 0 || dev >= kMaxDevices) return fail(SEIS_E_INVALID, "seis_forward_noalloc: device index out of range");
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_ptr[dev]) {
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr) return fail_cuda("cudaGetSymbolAddress", e);
        g_scratch_ptr[dev] = ptr;
    }
    *out = (unsigned char*)g_scratch_ptr[dev];
    return 0;
}

// vec and result must be memory of the current device: a host pointer handed to
// a kernel would fault (or, where the GPU can reach host memory, be used silently).
int require_device_memory(const void* p, int dev, const char* name)
{
    cudaPointerAttributes at{};
    cudaError_t e = cudaPointerGetAttributes(&at, p);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail_cuda("cudaPointerGetAttributes", e);
    }
    if ((at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged) || at.device != dev) {
        char msg[200];
        snprintf(msg, sizeof msg, "seis_forward_noalloc: %s must be device memory of the current device (%d)", name,
                 dev);
        return fail(SEIS_E_INVALID, msg);
    }
    return 0;
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
    if (G->nshots > kMaxShots || G->nrec > kMaxRec || G->nbc > kMaxNbc) {
        char msg[200];
        snprintf(msg, sizeof msg, "seis_forward_noalloc: at most %d shots, %d receivers and nbc %d", kMaxShots,
                 kMaxRec, kMaxNbc);
        return fail(SEIS_E_INVALID, msg);
    }
    const int NZ = G->nz + 2 * G->nbc, NX = G->nx + 2 * G->nbc;
    if ((long long)NZ * NX > (1LL << 28)) return fail(SEIS_E_INVALID, "seis_forward_noalloc: padded grid too large");
    for (int s = 0; s < G->nshots; ++s)
        if (G->src_z[s] < 0 || G->src_z[s] >= NZ || G->src_x[s] < 0 || G->src_x[s] >= NX)
            return fail(SEIS_E_INVALID, "seis_forward_noalloc: source outside the padded grid");
    for (int r = 0; r < G->nrec; ++r)
        if (G->rec_z[r] < 0 || G->rec_z[r] >= NZ || G->rec_x[r] < 0 || G->rec_x[r] >= NX)
            return fail(SEIS_E_INVALID, "seis_forward_noalloc: receiver outside the padded grid");
    std::vector<double> ricker;
    const int nw = host_ricker(G->freq, G->dt, G->nt, ricker);
    if (nw < 0) return fail(SEIS_E_INVALID, "seis_forward_noalloc: nt is smaller than the Ricker wavelet");
    if (nw > kMaxWavelet) {
        char msg[200];
        snprintf(msg, sizeof msg, "seis_forward_noalloc: the Ricker wavelet has %d samples, at most %d are supported",
                 nw, kMaxWavelet);
        return fail(SEIS_E_INVALID, msg);
    }

    GridDev g{};
    const int pitch = (NX + 31) / 32 * 32;
    g.NZ = NZ; g.NX = NX; g.pitch = pitch;
    g.xlo = G->nbc; g.xhi = G->nbc + G->nx;
    g.NP = (long long)NZ * pitch;
    g.nt = G->nt; g.nrec = G->nrec;
    const int tiles_x = (NX + kTX - 1) / kTX, tiles_z = (NZ + kTZ - 1) / kTZ, ntiles = tiles_x * tiles_z;
    const Layout L = layout_for(g.NP, pitch, NZ, G->nt, G->nshots, G->nrec, ntiles);
    if (L.total > kNoAllocScratchBytes) {
        char msg[300];
        snprintf(msg, sizeof msg,
                 "seis_forward_noalloc: this geometry needs %zu bytes of scratch; the no-allocation path holds %zu "
                 "(24 bytes per padded point at the row pitch plus 4*nt*nrec bytes of records and a few KB)",
                 L.total, kNoAllocScratchBytes);
        return fail(SEIS_E_INVALID, msg);
    }

    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail_cuda("cudaGetDevice", e);
    int rc = require_device_memory(vec, dev, "vec");
    if (!rc) rc = require_device_memory(result, dev, "result");
    if (rc) return rc;
    unsigned char* base = nullptr;
    if ((rc = scratch_address(dev, &base))) return rc;
    cudaStream_t st = (cudaStream_t)stream;

    // the geometry's constants, by value
    Consts c{};
    c.nshots = G->nshots; c.nrec = G->nrec; c.nbc = G->nbc; c.nw = nw; c.nz = G->nz; c.nx = G->nx;
    c.tiles_x = tiles_x; c.ntiles = ntiles;
    {
        std::vector<double> d1;
        host_damp_1d(G->nbc, G->dx, d1);
        for (int i = 0; i < G->nbc; ++i) c.d1[i] = (float)d1[i];
    }
    for (int k = 0; k < nw; ++k) c.wavelet[k] = ricker[k];
    for (int s = 0; s < G->nshots; ++s) { c.src_z[s] = G->src_z[s]; c.src_x[s] = G->src_x[s]; }
    for (int r = 0; r < G->nrec; ++r) { c.rec_z[r] = G->rec_z[r]; c.rec_x[r] = G->rec_x[r]; }
    noalloc_setup_kernel<<<1, 256, 0, st>>>(c, g, (float*)(base + L.dampx), (float*)(base + L.dampz),
                                            (double*)(base + L.ricker), (int*)(base + L.src_z),
                                            (int*)(base + L.src_x), (int*)(base + L.rec_off),
                                            (int*)(base + L.tstart), (int*)(base + L.tlist));

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
        e = cudaMemsetAsync(p, 0, sizeof(float) * 3 * g.NP, st);
        if (e == cudaSuccess) e = cudaMemsetAsync(u, 0, sizeof(float) * g.NP, st);
        if (e != cudaSuccess) return fail_cuda("cudaMemsetAsync", e);
        for (int t = 0; t < G->nt; ++t) fwd_step_kernel<false><<<grid, block, 0, st>>>(a, t);
        store_records_kernel<<<std::max(1, (int)std::min<long long>((per_shot + 255) / 256, 152 * 16)), 256, 0, st>>>(
            s, 1, per_shot, rec, result);
    }
    e = cudaGetLastError();
    return e == cudaSuccess ? 0 : fail_cuda("kernel launch", e);
}
