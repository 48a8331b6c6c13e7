// engine.cu -- SeisEngine: workspace, preparation / finalisation kernels,
// CUDA-graph sweeps and the C ABI declared in include/seis_gb300.h.
//
// Call flow of seis_vel_to_seis (the reference's vel_to_seis,
// core/seis_forward2.py:146-331, over many models at once):
//   prep_models      alpha, kappa factors (+ tangent) per model   prep_run(_diff) :333-359
//   per chunk of concurrently swept shot slots:
//     chunk_setup    slot -> (model, shot), s_mod / s_mod_diff    :205-208,253-254
//     forward graph  nt x fwd_step_kernel<TAN>                    :211-283
//     store_records  FP32 records -> caller's FP64 result         :249,283,320-323
//     adjoint:       seeds (residual or w), nt x adj_step_kernel,
//                    per-model FP64 accumulation                  :285-314
//   finalise         (2/v) Gv folded back to nz x nx, min_vel     prep_run_adjoint :361-377,
//                                                                  unpad_edge_padded_gradient
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/seis_gb300.h"
#include "errors.h"
#include "host_setup.h"
#include "cluster_kernels.cuh"
#include "tmem_sweeps.cuh"
#include "prep_kernels.cuh"
#include "sweep_kernels.cuh"
#include "wave_sweeps.cuh"

using namespace seis;

namespace {

thread_local std::string g_create_error;

}  // namespace

void seis::set_thread_error(const std::string& msg) { g_create_error = msg; }

// ---------------------------------------------------------------------------
// cluster kernel shapes
// ---------------------------------------------------------------------------

namespace {

constexpr int kClusterSP = 320;   // compile-time row pitches of the cluster kernels (NX + 4 <= pitch)
constexpr int kClusterSP2 = 384;
constexpr size_t kSmemLimit = 227 * 1024;

using ClusterKernel = void (*)(ClusterArgs);

// One instantiation of a cluster sweep: C CTAs per cluster, strips of RPT
// rows, W columns per thread, at most `threads` threads per CTA.  Rows per band
// R = ceil(NZ / C) (with column pairs, rounded up to whole strips), one strip
// per group of SP / W threads.  For the 70x70 models' 310-row grids: 640
// threads as 2 groups of 320 one-column threads or 4 groups of 160 pair
// threads.  (640 threads = 5 warps per scheduler at up to 96 registers: 320
// threads with twice the rows per thread, or 800 threads at 72 registers, were
// both slower on GB300.)
struct ClusterShape {
    bool adjoint;
    int C, RPT, W, threads;
    int sp;            // compile-time row pitch: grids whose pitch is sp and NX + 4 <= sp
    bool alpha_smem;   // forward: alpha of the band in shared memory instead of registers
    bool tangent;      // forward sweep that also advances the tangent field
    bool shuffle;      // horizontal neighbours by warp shuffles instead of shared loads
    bool tmem;         // adjoint with alpha, the gradient sums and the carried history level in tensor memory
    ClusterKernel kernel;
};
#define SEIS_FWD(C_, RPT_, W_, T_, AS_) \
    {false, C_, RPT_, W_, T_, kClusterSP, AS_, false, false, false, \
     fwd_cluster_kernel<C_, RPT_, W_, kClusterSP, T_, AS_, false>}
#define SEIS_FWD_SH(C_, RPT_, W_, T_, AS_) \
    {false, C_, RPT_, W_, T_, kClusterSP, AS_, false, true, false, \
     fwd_cluster_kernel<C_, RPT_, W_, kClusterSP, T_, AS_, false, true>}
#define SEIS_TAN(C_, RPT_, W_, T_) \
    {false, C_, RPT_, W_, T_, kClusterSP, false, true, false, false, \
     fwd_cluster_kernel<C_, RPT_, W_, kClusterSP, T_, false, true>}
#define SEIS_ADJ(C_, RPT_, W_, T_) \
    {true, C_, RPT_, W_, T_, kClusterSP, true, false, false, false, adj_cluster_kernel<C_, RPT_, W_, kClusterSP, T_>}
#define SEIS_FWD_TM(C_, RPT_, T_, SP_) \
    {false, C_, RPT_, 2, T_, SP_, false, false, false, true, fwd_cluster_tm_kernel<C_, RPT_, SP_, T_>}
#define SEIS_TAN_TM(C_, RPT_, T_) \
    {false, C_, RPT_, 2, T_, kClusterSP, false, true, false, true, tan_cluster_tm_kernel<C_, RPT_, kClusterSP, T_>}
#define SEIS_ADJ_TM(C_, RPT_, T_, SP_) \
    {true, C_, RPT_, 2, T_, SP_, false, false, false, true, adj_cluster_tm_kernel<C_, RPT_, SP_, T_>}
const ClusterShape kShapes[] = {
    SEIS_FWD(8, 20, 1, 640, true), SEIS_FWD(16, 10, 1, 640, false), SEIS_FWD(8, 10, 2, 640, true),
    SEIS_FWD(16, 5, 2, 640, false), SEIS_FWD(10, 16, 1, 640, true), SEIS_FWD(10, 8, 2, 640, true),
    SEIS_FWD_SH(10, 8, 2, 640, true),  SEIS_FWD_TM(10, 8, 640, kClusterSP),
    SEIS_TAN(16, 10, 1, 640),       SEIS_TAN(16, 5, 2, 640),      SEIS_TAN_TM(16, 5, 640),
    SEIS_ADJ(16, 10, 1, 640),       SEIS_ADJ(16, 5, 2, 640),      SEIS_ADJ_TM(10, 8, 640, kClusterSP),
    SEIS_ADJ_TM(10, 11, 480, kClusterSP),
    // grids of pitch 384 (padded widths 353..380, e.g. 100x140 models with nbc = 120): the
    // tensor-memory forward on 10-CTA clusters (34- to 36-row bands, 3 strips of 12 rows of
    // 192 column-pair threads) and adjoint on 16-CTA clusters (22-row bands)
    SEIS_FWD_TM(10, 12, 576, kClusterSP2), SEIS_ADJ_TM(16, 8, 576, kClusterSP2),
};
#undef SEIS_TAN
#undef SEIS_FWD
#undef SEIS_FWD_SH
#undef SEIS_ADJ
#undef SEIS_ADJ_TM
#undef SEIS_FWD_TM
#undef SEIS_TAN_TM
constexpr int kNumShapes = (int)(sizeof(kShapes) / sizeof(kShapes[0]));

// Throughput per SM of a cluster sweep over the two-step tiled sweep on 70x70
// models, measured on GB300 (forward, adjoint, forward + tangent): 6.2 / 1.91,
// 4.16 / 1.1 and 2.47 / 0.99 G point-steps/s per SM.  They size the side sweeps.
constexpr double kFwdClusterOverTiled = 3.24;
constexpr double kAdjClusterOverTiled = 3.8;
constexpr double kAdjTmClusterOverTiled = 4.7;   // the 10-CTA tensor-memory adjoint: 5.2 / 1.1
constexpr double kTanClusterOverTiled = 2.5;
// One shot's forward on an 8-CTA cluster (register sweep, alpha in shared memory) over one
// round of the 10-CTA tensor-memory forward, measured on GB300 with both running at once:
// 1.81 / 1.40 ms.  It sizes the forward side slots when they run on 8-CTA clusters.
constexpr double kFwdSide8OverTm = 1.29;

}  // namespace

// ---------------------------------------------------------------------------
// engine
// ---------------------------------------------------------------------------

struct SeisEngine {
    // geometry
    int nz = 0, nx = 0, nbc = 0, nt = 0, nshots = 0, nrec = 0;
    double dx = 0, dt = 0, freq = 0;
    std::vector<int> src_z, src_x, rec_z, rec_x;
    GridDev g{};
    ModelGeom mg{};
    int tiles_x = 0, tiles_z = 0;
    int max_models = 0, slots = 0;

    // cluster-resident sweeps (cluster_kernels.cuh): applicability and launch
    // shape of each instantiation in kShapes
    struct ClusterPlan {
        bool ok = false;
        const ClusterShape* shape = nullptr;
        int C = 0, R = 0, G = 0, threads = 0, nclusters = 0;
        int W = 1;            // columns per thread
        size_t smem = 0;
    } plans[kNumShapes];
    int cols = 2;             // preferred columns per thread of the cluster sweeps (1 or 2)
    int shuffle = 0;          // forward: horizontal neighbours by warp shuffles (where a shape has them)
    int adj_cluster = 0;      // CTAs per cluster of the cluster adjoint (0 automatic, 10 or 16)
    int adj_rows = 0;         // rows per thread of the tensor-memory adjoint (0 automatic: 8, or 11)
    int fwd_tmem = 1;         // forward: alpha in tensor memory (where a shape has it: 10-CTA, column pairs)
    int path = 0;             // 0 auto, 1 tiled per-step sweeps only, 2 cluster sweeps required
    int fwd_cluster = 0;      // CTAs per cluster of the forward sweep (0 automatic, 8, 10 or 16)
    int skip_copy_level = -1; // test hook of the adjoint's bounded waits (see seis_set_option)
    int adj_fuse = 1;         // tiled adjoint: two steps per launch where the grid allows it
    int adj_hoist = 4;        // two-step tiled adjoint: rows of a thread whose loads are issued together
    int fwd_fuse = 1;         // tiled forward (no tangent): two steps per launch likewise
    int adj_side = -1;        // slots of a chunk whose adjoint runs tiled beside the cluster adjoint
                              // (-1 automatic, 0 none)
    int fwd_side = -1;        // likewise for the forward (and tangent) sweep
    int fwd_side_cluster = -1;// forward side slots: 0 tiled sweep, C > 0 a concurrent C-CTA cluster sweep of
                              // fwd_side_clusters clusters on the SMs the main clusters leave free, -1
                              // automatic (8 where the 10-CTA main clusters leave 16 SMs free)
    int fwd_side_clusters = 2;
    int num_sms = 0;
    int* d_err = nullptr;     // device error word of the cluster sweeps: sticky (bits OR-ed in by every
                              // call) until seis_device_status reports and clears it
    int* h_err = nullptr;     // pinned host mirror of d_err, copied at the end of every call (read
                              // without a sync through seis_get_info "err_word" once the stream is done)
    // sweep kernel launches and path (1 tiled, 2 cluster) of the last call
    long long last_fwd_launches = 0, last_adj_launches = 0;
    int last_fwd_path = 0, last_adj_path = 0;
    int last_adj_side = 0;    // slots of the last call's chunks that ran the side adjoint
    int last_fwd_side = 0;    // ... the side forward
    cudaStream_t last_stream = nullptr;

    // constant device data
    float* d_dampx = nullptr;
    float* d_dampz = nullptr;
    double* d_dampx64 = nullptr;
    double* d_dampz64 = nullptr;
    double* d_ricker = nullptr;
    int* d_src_z = nullptr;
    int* d_src_x = nullptr;
    int* d_rec_off = nullptr;
    int* d_rec_z = nullptr;
    int* d_rec_x = nullptr;
    int* d_tile_rec_start = nullptr;
    int* d_tile_rec_list = nullptr;

    // per model
    float* d_alpha = nullptr;
    float* d_kfac = nullptr;
    float* d_alpha_d = nullptr;
    float* d_kdfac = nullptr;
    double* d_acc_v = nullptr;
    double* d_acc_k = nullptr;

    // per slot
    ShotDesc* d_shots = nullptr;
    float* d_p = nullptr;
    float* d_uring = nullptr;
    float* d_uhist = nullptr;
    float* d_dp = nullptr;
    float* d_du = nullptr;
    float* d_smod = nullptr;
    float* d_smod_d = nullptr;
    float* d_rec = nullptr;
    float* d_drec = nullptr;
    float* d_lam = nullptr;
    float* d_mu = nullptr;
    float* d_gv = nullptr;
    float* d_gk = nullptr;
    float* d_seed = nullptr;

    // graphs: forward [tan][hist], adjoint
    cudaGraphExec_t fwd_graph[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    cudaGraphExec_t adj_graph = nullptr;
    // checkpointed adjoint (every ck steps): forward with checkpoint saves [tan],
    // adjoint with per-segment restore + recompute; built for ck_graph_k
    int ck = 0, ck_graph_k = 0;
    cudaGraphExec_t ck_fwd_graph[2] = {nullptr, nullptr};
    cudaGraphExec_t ck_adj_graph = nullptr;
    float* d_ckp = nullptr;    // [slot][ncp][NP] p_{t0+1} at t0 = 0, k, 2k, ...
    float* d_cku = nullptr;    // [slot][ncp][NP] u_{t0+1}
    float* d_ring = nullptr;   // [slot][k+1][NP] increments of one segment
    size_t ck_alloc_k = 0;
    cudaStream_t cap_stream = nullptr;

    // host buffers of a call: device staging (max_models wide, allocated on first
    // use), a copy stream, and the call's host destinations of per-chunk records
    double* d_in_vec = nullptr;
    double* d_in_vd = nullptr;
    double* d_in_va = nullptr;
    double* d_out_res = nullptr;
    double* d_out_rd = nullptr;
    double* d_out_ra = nullptr;
    double* d_out_mf = nullptr;
    cudaStream_t io_stream = nullptr;
    cudaEvent_t io_ev = nullptr;       // ordering point between the call stream and io_stream
    cudaEvent_t io_in_ev = nullptr;    // vec_adjoint uploaded
    // side sweeps: the cluster sweep on a high-priority stream, the tiled side sweep
    // of the chunk's last slots on a low-priority one, forked from and joined back
    // into the call's stream
    cudaStream_t hi_stream = nullptr, side_stream = nullptr;
    cudaEvent_t fork_ev = nullptr, join_hi_ev = nullptr, join_side_ev = nullptr;
    // captured tiled side sweeps by split (first slot s0, ns slots): the side adjoint, and
    // the side forward [tan][hist]; a few splits each (automatic splits follow each
    // chunk's shot count)
    struct SideGraph {
        int s0, ns;
        cudaGraphExec_t g;
    };
    std::vector<SideGraph> adj_side_graphs;
    std::vector<SideGraph> fwd_side_graphs[2][2];
    struct HostIO {
        bool wait_va = false;          // wait for io_in_ev before the first use of vec_adjoint
        double* res = nullptr;         // host destinations (nullptr: device output)
        double* rd = nullptr;
    } io;

    // statistics
    long long launches = 0, fwd_step_launches = 0, adj_step_launches = 0;
    std::vector<cudaEvent_t> ev_pool;
    std::vector<std::pair<int, int>> fwd_ev, adj_ev;  // indices into ev_pool for the last call
    std::vector<std::pair<int, int>> adj_cl_ev;       // the cluster adjoint launch of each chunk

    // persistent wavefront sweeps (sweep_path 3; wave_sweeps.cuh)
    struct WaveBlob {
        std::string bytes;              // host image
        void* d = nullptr;              // device copy
        cudaEvent_t ready = nullptr;    // its upload
    };
    std::vector<WaveBlob> wave_blobs;   // programs and group tables, uploaded once each
    int* d_wave_progress = nullptr;     // [slots][tiles] stages completed
    unsigned long long* d_wave_state = nullptr;   // [0] dequeue counter, [1] abort flag
    int wave_group_slots = 0;           // slots per group (0 automatic)
    int wave_fwd_blocks = 4;            // register budget of the forward kernel (resident blocks per SM)
    int wave_resident[9] = {};          // resident blocks of each kernel (0: not queried)

    std::mutex mu;
    std::string err;

    int fail(int code, const char* fmt, ...)
    {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        err = buf;
        return code;
    }
};

namespace {

#define CK(call)                                                                                    \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess)                                                                      \
            return E->fail(e_ == cudaErrorMemoryAllocation ? SEIS_E_NOMEM : SEIS_E_CUDA,            \
                           "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

template <class T>
int dalloc(SeisEngine* E, T** p, size_t n)
{
    if (*p) return 0;
    CK(cudaMalloc((void**)p, sizeof(T) * (n ? n : 1)));
    return 0;
}

template <class T>
void dfree(T*& p)
{
    if (p) cudaFree(p);
    p = nullptr;
}

// Executable graphs of side sweeps (an in-flight graph is freed when it completes).
void destroy_graphs(std::vector<SeisEngine::SideGraph>& v)
{
    for (auto& e : v)
        if (e.g) cudaGraphExecDestroy(e.g);
    v.clear();
}

void destroy_side_graphs(SeisEngine* E)
{
    destroy_graphs(E->adj_side_graphs);
    for (auto& row : E->fwd_side_graphs)
        for (auto& v : row) destroy_graphs(v);
}

void free_all(SeisEngine* E)
{
    for (auto& row : E->fwd_graph)
        for (auto& gexec : row)
            if (gexec) { cudaGraphExecDestroy(gexec); gexec = nullptr; }
    if (E->adj_graph) { cudaGraphExecDestroy(E->adj_graph); E->adj_graph = nullptr; }
    for (auto& gexec : E->ck_fwd_graph)
        if (gexec) { cudaGraphExecDestroy(gexec); gexec = nullptr; }
    if (E->ck_adj_graph) { cudaGraphExecDestroy(E->ck_adj_graph); E->ck_adj_graph = nullptr; }
    dfree(E->d_ckp); dfree(E->d_cku); dfree(E->d_ring);
    if (E->cap_stream) { cudaStreamDestroy(E->cap_stream); E->cap_stream = nullptr; }
    if (E->io_stream) { cudaStreamDestroy(E->io_stream); E->io_stream = nullptr; }
    if (E->io_ev) { cudaEventDestroy(E->io_ev); E->io_ev = nullptr; }
    if (E->io_in_ev) { cudaEventDestroy(E->io_in_ev); E->io_in_ev = nullptr; }
    destroy_side_graphs(E);
    if (E->hi_stream) { cudaStreamDestroy(E->hi_stream); E->hi_stream = nullptr; }
    if (E->side_stream) { cudaStreamDestroy(E->side_stream); E->side_stream = nullptr; }
    for (cudaEvent_t* ev : {&E->fork_ev, &E->join_hi_ev, &E->join_side_ev})
        if (*ev) { cudaEventDestroy(*ev); *ev = nullptr; }
    dfree(E->d_in_vec); dfree(E->d_in_vd); dfree(E->d_in_va);
    dfree(E->d_out_res); dfree(E->d_out_rd); dfree(E->d_out_ra); dfree(E->d_out_mf);
    for (auto ev : E->ev_pool) cudaEventDestroy(ev);
    E->ev_pool.clear();
    dfree(E->d_dampx); dfree(E->d_dampz); dfree(E->d_dampx64); dfree(E->d_dampz64); dfree(E->d_ricker);
    dfree(E->d_src_z); dfree(E->d_src_x); dfree(E->d_rec_off); dfree(E->d_rec_z); dfree(E->d_rec_x); dfree(E->d_tile_rec_start);
    dfree(E->d_tile_rec_list); dfree(E->d_alpha); dfree(E->d_kfac); dfree(E->d_alpha_d); dfree(E->d_kdfac);
    dfree(E->d_acc_v); dfree(E->d_acc_k); dfree(E->d_shots); dfree(E->d_p); dfree(E->d_uring);
    dfree(E->d_uhist); dfree(E->d_dp); dfree(E->d_du); dfree(E->d_smod); dfree(E->d_smod_d); dfree(E->d_rec);
    dfree(E->d_drec); dfree(E->d_lam); dfree(E->d_mu); dfree(E->d_gv); dfree(E->d_gk); dfree(E->d_seed);
    for (auto& b : E->wave_blobs) {
        if (b.d) cudaFree(b.d);
        if (b.ready) cudaEventDestroy(b.ready);
    }
    E->wave_blobs.clear();
    dfree(E->d_wave_progress);
    dfree(E->d_wave_state);
    dfree(E->d_err);
    if (E->h_err) { cudaFreeHost(E->h_err); E->h_err = nullptr; }
}

int grid_blocks(long long n, int threads)
{
    long long b = (n + threads - 1) / threads;
    return (int)std::max(1LL, std::min(b, 152LL * 16));
}

FwdArgs make_fwd_args(SeisEngine* E, bool tan, bool hist, float* u_override = nullptr, int ulevels_override = 0)
{
    FwdArgs a{};
    a.g = E->g;
    a.shots = E->d_shots;
    a.alpha = E->d_alpha;
    a.kfac = E->d_kfac;
    a.alpha_d = E->d_alpha_d;
    a.kdfac = E->d_kdfac;
    a.dampx = E->d_dampx;
    a.dampz = E->d_dampz;
    a.p = E->d_p;
    a.u = hist ? E->d_uhist : E->d_uring;
    a.ulevels = hist ? E->nt + 1 : 3;
    if (u_override) {
        a.u = u_override;
        a.ulevels = ulevels_override;
    }
    a.u_slot_stride = (long long)a.ulevels * E->g.NP;
    a.dp = E->d_dp;
    a.du = E->d_du;
    a.smod = E->d_smod;
    a.smod_d = E->d_smod_d;
    a.rec = E->d_rec;
    a.drec = E->d_drec;
    a.tile_rec_start = E->d_tile_rec_start;
    a.tile_rec_list = E->d_tile_rec_list;
    a.rec_off = E->d_rec_off;
    (void)tan;
    return a;
}

AdjArgs make_adj_args(SeisEngine* E)
{
    AdjArgs a{};
    a.g = E->g;
    a.shots = E->d_shots;
    a.alpha = E->d_alpha;
    a.kfac = E->d_kfac;
    a.dampx = E->d_dampx;
    a.dampz = E->d_dampz;
    a.u = E->d_uhist;
    a.ulevels = E->nt + 1;
    a.u_slot_stride = (long long)(E->nt + 1) * E->g.NP;
    a.lam = E->d_lam;
    a.mu = E->d_mu;
    a.gv = E->d_gv;
    a.gk = E->d_gk;
    a.seed = E->d_seed;
    a.tile_rec_start = E->d_tile_rec_start;
    a.tile_rec_list = E->d_tile_rec_list;
    a.rec_off = E->d_rec_off;
    return a;
}

// Can the tiled forward take two steps per launch here?
bool fwd_fused(const SeisEngine* E)
{
    return E->fwd_fuse && E->g.NX % 2 == 0 && E->g.NX >= kFW && E->g.NZ >= kFH;
}

// Launches of steps t0 .. t1-1 taken in pairs (fuse) or one by one.
long long step_launches(bool fuse, int t0, int t1)
{
    const int n = t1 - t0;
    return fuse ? n / 2 + n % 2 : n;
}

// Step launches of a whole forward (fwd) or adjoint sweep of the tiled path; the
// checkpointed adjoint counts its recomputed forward segments too.
long long sweep_step_launches(const SeisEngine* E, bool fwd, bool ckmode);

// Forward steps t0 .. t1-1 (with or without the tangent): pairs where possible.
void launch_fwd_steps(SeisEngine* E, const FwdArgs& a, bool tan, int t0, int t1, cudaStream_t st, int nslots = 0)
{
    const dim3 grid(E->tiles_x, E->tiles_z, nslots ? nslots : E->slots), block(kBX, kBZ);
    const bool fuse = fwd_fused(E);
    for (int t = t0; t < t1;) {
        if (fuse && t + 1 < t1) {
            if (tan) fwd_step2_kernel<true><<<grid, block, fused_fwd_smem<true>(), st>>>(a, t);
            else fwd_step2_kernel<false><<<grid, block, fused_fwd_smem<false>(), st>>>(a, t);
            t += 2;
        } else {
            if (tan) fwd_step_kernel<true><<<grid, block, 0, st>>>(a, t);
            else fwd_step_kernel<false><<<grid, block, 0, st>>>(a, t);
            t += 1;
        }
    }
}

// Capture nt step launches on `st` into an executable graph.
int capture_fwd(SeisEngine* E, bool tan, bool hist, cudaStream_t st, cudaGraphExec_t* out)
{
    const FwdArgs a = make_fwd_args(E, tan, hist);
    cudaGraph_t graph = nullptr;
    CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    launch_fwd_steps(E, a, tan, 0, E->nt, st);
    cudaError_t e = cudaStreamEndCapture(st, &graph);
    if (e != cudaSuccess) return E->fail(SEIS_E_CUDA, "forward sweep capture failed: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(out, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return E->fail(SEIS_E_CUDA, "forward graph instantiate failed: %s", cudaGetErrorString(e));
    return 0;
}

// Can the tiled adjoint take two steps per launch here?  (Column pairs need an
// even width; the staged tile with its 4-cell halo must not wrap onto itself.)
bool adj_fused(const SeisEngine* E)
{
    return E->adj_fuse && E->g.NX % 2 == 0 && E->g.NX >= kFW && E->g.NZ >= kFH;
}

// Reverse steps t1-1 .. t0 of the tiled adjoint: pairs of steps per launch where possible
// (over nslots slots from the args' first; 0 = all of the chunk's slots).
void launch_adj_steps(SeisEngine* E, const AdjArgs& a, int t0, int t1, cudaStream_t st, int nslots = 0)
{
    const dim3 grid(E->tiles_x, E->tiles_z, nslots ? nslots : E->slots), block(kBX, kBZ);
    const bool fuse = adj_fused(E);
    for (int t = t1 - 1; t >= t0;) {
        if (fuse && t - 1 >= t0) {
            auto k = E->adj_hoist == 4 ? adj_step2_kernel<4> : (E->adj_hoist == 2 ? adj_step2_kernel<2>
                                                                                   : adj_step2_kernel<1>);
            k<<<grid, block, kFusedAdjSmem, st>>>(a, t);
            t -= 2;
        } else {
            adj_step_kernel<<<grid, block, 0, st>>>(a, t);
            t -= 1;
        }
    }
}

long long sweep_step_launches(const SeisEngine* E, bool fwd, bool ckmode)
{
    const bool ff = fwd_fused(E), af = adj_fused(E);
    if (!ckmode) return fwd ? step_launches(ff, 0, E->nt) : step_launches(af, 0, E->nt);
    long long n = 0;
    for (int t0 = 0; t0 < E->nt; t0 += E->ck) {
        const int t1 = std::min(t0 + E->ck, E->nt);
        n += fwd ? step_launches(ff, t0, t1) : step_launches(ff, t0, t1) + step_launches(af, t0, t1);
    }
    return n;
}

int capture_adj(SeisEngine* E, cudaStream_t st, cudaGraphExec_t* out)
{
    const AdjArgs a = make_adj_args(E);
    cudaGraph_t graph = nullptr;
    CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    launch_adj_steps(E, a, 0, E->nt, st);
    cudaError_t e = cudaStreamEndCapture(st, &graph);
    if (e != cudaSuccess) return E->fail(SEIS_E_CUDA, "adjoint sweep capture failed: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(out, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return E->fail(SEIS_E_CUDA, "adjoint graph instantiate failed: %s", cudaGetErrorString(e));
    return 0;
}

// The tiled forward (tangent, history) over slots s0 .. s0+ns-1 only: the side sweep
// beside the cluster forward, the slot arrays offset to the first slot.
int capture_fwd_side(SeisEngine* E, bool tan, bool hist, int s0, int ns, cudaStream_t st, cudaGraphExec_t* out)
{
    FwdArgs a = make_fwd_args(E, tan, hist);
    const long long NP = E->g.NP, per_shot = (long long)E->nt * E->nrec;
    a.shots += s0;
    a.p += (long long)s0 * 3 * NP;
    a.u += (long long)s0 * a.u_slot_stride;
    a.smod += (long long)s0 * E->nt;
    a.rec += (long long)s0 * per_shot;
    if (tan) {
        a.dp += (long long)s0 * 3 * NP;
        a.du += (long long)s0 * 3 * NP;
        a.smod_d += (long long)s0 * E->nt;
        a.drec += (long long)s0 * per_shot;
    }
    cudaGraph_t graph = nullptr;
    CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    launch_fwd_steps(E, a, tan, 0, E->nt, st, ns);
    cudaError_t e = cudaStreamEndCapture(st, &graph);
    if (e != cudaSuccess) return E->fail(SEIS_E_CUDA, "side forward capture failed: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(out, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return E->fail(SEIS_E_CUDA, "side forward instantiate failed: %s", cudaGetErrorString(e));
    return 0;
}

// Side sweep split of a chunk of S slots for a cluster plan: the cluster launch takes
// whole rounds of its resident clusters (r rounds, r * ncl slots) and the last `ns`
// slots run the tiled sweep on the SMs the clusters leave free.  `ratio` is the
// cluster kernel's throughput per SM over the tiled kernel's (measured on GB300), so
// that one side slot takes rho = ratio * C / idle_SMs cluster rounds; r minimises
// max(r, rho * (S - r * ncl)).  option: -1 automatic, 0 none, n > 0 exactly n slots.
void side_split(const SeisEngine* E, const SeisEngine::ClusterPlan& P, int S, int option, double ratio, int* s0,
                int* ns)
{
    *s0 = S;
    *ns = 0;
    int side = option;
    if (option < 0) {
        side = 0;
        const int ncl = std::max(1, P.nclusters);
        const int idle = E->num_sms - ncl * P.C;
        if (idle <= 0 || S < ncl) return;
        const double rho = ratio * P.C / idle;
        const double rc = rho * S / (1.0 + rho * ncl);
        double best = std::ceil((double)S / ncl);     // all slots on the clusters
        for (int r : {(int)std::floor(rc), (int)std::ceil(rc)}) {
            r = std::min(std::max(r, 1), S / ncl);
            const double t = std::max((double)r, rho * (S - r * ncl));
            if (t < best) {
                best = t;
                side = S - r * ncl;
            }
        }
    }
    if (side > 0 && side < S) {
        *s0 = S - side;
        *ns = side;
    }
}

// The tiled adjoint over slots s0 .. s0+ns-1 only (the side sweep that runs beside the
// cluster adjoint on the SMs its clusters leave free): the same kernels, their slot
// arrays offset to the first slot.
int capture_adj_side(SeisEngine* E, int s0, int ns, cudaStream_t st, cudaGraphExec_t* out)
{
    AdjArgs a = make_adj_args(E);
    const long long NP = E->g.NP;
    a.shots += s0;
    a.u += (long long)s0 * a.u_slot_stride;
    a.lam += (long long)s0 * 3 * NP;
    a.mu += (long long)s0 * 3 * NP;
    a.gv += (long long)s0 * NP;
    a.gk += (long long)s0 * NP;
    a.seed += (long long)s0 * E->nt * E->nrec;
    cudaGraph_t graph = nullptr;
    CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    launch_adj_steps(E, a, 0, E->nt, st, ns);
    cudaError_t e = cudaStreamEndCapture(st, &graph);
    if (e != cudaSuccess) return E->fail(SEIS_E_CUDA, "side adjoint capture failed: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(out, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return E->fail(SEIS_E_CUDA, "side adjoint instantiate failed: %s", cudaGetErrorString(e));
    return 0;
}

// Checkpointed sweeps (k = E->ck): the forward saves (p_{t+1}, u_{t+1}) at
// t = 0, k, 2k, ... and keeps u in a ring of k+1 levels; the adjoint restores
// each segment's checkpoint, recomputes its k forward steps into the ring
// and runs the segment's adjoint steps from it, last segment first.  The
// recomputed increments are bitwise those of the first forward sweep.
void launch_slot_copy(SeisEngine* E, long long n, const float* src, long long ss, float* dst, long long ds,
                      cudaStream_t st)
{
    const dim3 grid((unsigned)std::min<long long>((n + 255) / 256, 64), (unsigned)E->slots);
    slot_copy_kernel<<<grid, 256, 0, st>>>(E->d_shots, n, src, ss, dst, ds);
}

int capture_ck_fwd(SeisEngine* E, bool tan, cudaStream_t st, cudaGraphExec_t* out)
{
    const int k = E->ck, L = k + 1;
    const long long NP = E->g.NP;
    const int ncp = (E->nt + k - 1) / k;
    const FwdArgs a = make_fwd_args(E, tan, false, E->d_ring, L);
    cudaGraph_t graph = nullptr;
    CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    for (int c = 0; c < ncp; ++c) {
        const int t0 = c * k, t1 = std::min(t0 + k, E->nt);
        launch_slot_copy(E, NP, E->d_p + (long long)((t0 + 1) % 3) * NP, 3 * NP, E->d_ckp + (long long)c * NP,
                         (long long)ncp * NP, st);
        launch_slot_copy(E, NP, E->d_ring + (long long)(t0 % L) * NP, (long long)L * NP,
                         E->d_cku + (long long)c * NP, (long long)ncp * NP, st);
        launch_fwd_steps(E, a, tan, t0, t1, st);
    }
    cudaError_t e = cudaStreamEndCapture(st, &graph);
    if (e != cudaSuccess) return E->fail(SEIS_E_CUDA, "checkpointed forward capture failed: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(out, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return E->fail(SEIS_E_CUDA, "checkpointed forward instantiate failed: %s", cudaGetErrorString(e));
    return 0;
}

int capture_ck_adj(SeisEngine* E, cudaStream_t st, cudaGraphExec_t* out)
{
    const int k = E->ck, L = k + 1;
    const long long NP = E->g.NP;
    const int ncp = (E->nt + k - 1) / k;
    const FwdArgs f = make_fwd_args(E, false, false, E->d_ring, L);
    AdjArgs a = make_adj_args(E);
    a.u = E->d_ring;
    a.ulevels = L;
    a.u_slot_stride = (long long)L * NP;
    cudaGraph_t graph = nullptr;
    CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    for (int c = ncp - 1; c >= 0; --c) {
        const int t0 = c * k, t1 = std::min(t0 + k, E->nt);
        launch_slot_copy(E, NP, E->d_ckp + (long long)c * NP, (long long)ncp * NP,
                         E->d_p + (long long)((t0 + 1) % 3) * NP, 3 * NP, st);
        launch_slot_copy(E, NP, E->d_cku + (long long)c * NP, (long long)ncp * NP,
                         E->d_ring + (long long)(t0 % L) * NP, (long long)L * NP, st);
        launch_fwd_steps(E, f, false, t0, t1, st);
        launch_adj_steps(E, a, t0, t1, st);
    }
    cudaError_t e = cudaStreamEndCapture(st, &graph);
    if (e != cudaSuccess) return E->fail(SEIS_E_CUDA, "checkpointed adjoint capture failed: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(out, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return E->fail(SEIS_E_CUDA, "checkpointed adjoint instantiate failed: %s", cudaGetErrorString(e));
    return 0;
}

// ---------------------------------------------------------------------------
// persistent wavefront sweeps: one launch per sweep over groups of shot slots, of one
// engine (sweep_path 3) or of several (seis_vel_to_seis_multi)
// ---------------------------------------------------------------------------

// Device copy of a constant blob (a sweep program or a group table): uploaded once, in
// the stream order of its first use, and kept (up to kMaxWaveBlobs of them); every user
// waits for its upload event.  An engine's calls are ordered on their stream, as its
// workspace requires, so its blobs are read only by launches on that stream.
constexpr size_t kMaxWaveBlobs = 256;
constexpr size_t kMaxSideGraphs = 8;   // cached side-sweep graphs per kind
const void* wave_blob(SeisEngine* E, const std::string& bytes, cudaStream_t st, int* rc)
{
    *rc = 0;
    for (auto& b : E->wave_blobs)
        if (b.bytes == bytes) {
            cudaError_t e = cudaStreamWaitEvent(st, b.ready, 0);
            if (e != cudaSuccess) *rc = E->fail(SEIS_E_CUDA, "wave blob wait: %s", cudaGetErrorString(e));
            return b.d;
        }
    if (E->wave_blobs.size() >= kMaxWaveBlobs) {
        // many distinct batch shapes: drop the cached tables once this stream's launches,
        // the only ones of this engine that can still read them, have finished
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            *rc = E->fail(SEIS_E_CUDA, "wave blob cache: %s", cudaGetErrorString(e));
            return nullptr;
        }
        for (auto& old : E->wave_blobs) {
            cudaFree(old.d);
            cudaEventDestroy(old.ready);
        }
        E->wave_blobs.clear();
    }
    SeisEngine::WaveBlob b;
    b.bytes = bytes;
    cudaError_t e = cudaMalloc(&b.d, std::max<size_t>(bytes.size(), 16));
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b.ready, cudaEventDisableTiming);
    // from pageable memory: the source is staged before the call returns
    if (e == cudaSuccess) e = cudaMemcpyAsync(b.d, bytes.data(), bytes.size(), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaEventRecord(b.ready, st);
    if (e != cudaSuccess) {
        if (b.d) cudaFree(b.d);
        if (b.ready) cudaEventDestroy(b.ready);
        *rc = E->fail(e == cudaErrorMemoryAllocation ? SEIS_E_NOMEM : SEIS_E_CUDA, "wave blob upload: %s",
                      cudaGetErrorString(e));
        return nullptr;
    }
    E->wave_blobs.push_back(std::move(b));
    return E->wave_blobs.back().d;
}

// The wavefront kernel of a mode: forward (with the register budget of 4, 5 or 6 resident
// blocks per SM, E->wave_fwd_blocks), forward + tangent (3), reverse (4; 5 is slower on
// 70x70 and 350x500 grids, as it is for adj_step2_kernel).
template <int MODE>
using WaveKernel = void (*)(const WaveParams<MODE>);
template <int MODE>
WaveKernel<MODE> wave_kernel(const SeisEngine* E)
{
    if constexpr (MODE == 1) return wave_sweep_kernel<1, 3>;
    else if constexpr (MODE == 2) return wave_sweep_kernel<2, 4>;
    else
        return E->wave_fwd_blocks == 4 ? wave_sweep_kernel<0, 4>
                                       : (E->wave_fwd_blocks == 6 ? wave_sweep_kernel<0, 6> : wave_sweep_kernel<0, 5>);
}

int wave_slot(const SeisEngine* E, int mode) { return mode == 0 ? 2 + E->wave_fwd_blocks : mode; }   // 1, 2, 6, 7, 8

template <int MODE>
int wave_resident_t(SeisEngine* E)
{
    int& res = E->wave_resident[wave_slot(E, MODE)];
    if (!res) {
        WaveKernel<MODE> k = wave_kernel<MODE>(E);
        CK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, wave_smem<MODE>()));
        int b = 0;
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k, kThreads, wave_smem<MODE>()));
        if (b < 1) return E->fail(SEIS_E_CUDA, "wavefront sweep kernel (mode %d) cannot be resident", MODE);
        res = b * E->num_sms;
    }
    return 0;
}

int wave_resident_mode(SeisEngine* E, int mode)
{
    return mode == 0 ? wave_resident_t<0>(E) : (mode == 1 ? wave_resident_t<1>(E) : wave_resident_t<2>(E));
}

int wave_resident_of(const SeisEngine* E, int mode) { return E->wave_resident[wave_slot(E, mode)]; }

// One engine's sweep arguments in a launch's kernel parameters.
struct WaveArgs {
    FwdArgs f;
    AdjArgs a;
};

void wave_steps_fwd(const SeisEngine* E, std::vector<WaveStage>& v, int t0, int t1)
{
    const bool fuse = fwd_fused(E);
    for (int t = t0; t < t1;) {
        const bool two = fuse && t + 1 < t1;
        v.push_back({two ? kWaveF2 : kWaveF1, t, 0, 0});
        t += two ? 2 : 1;
    }
}

void wave_steps_adj(const SeisEngine* E, std::vector<WaveStage>& v, int t0, int t1)
{
    const bool fuse = adj_fused(E);
    for (int t = t1 - 1; t >= t0;) {
        const bool two = fuse && t - 1 >= t0;
        v.push_back({two ? kWaveA2 : kWaveA1, t, 0, 0});
        t -= two ? 2 : 1;
    }
}

// The stages of one sweep, in the order of the step launches of the graph path
// (capture_fwd / capture_adj, and capture_ck_fwd / capture_ck_adj with checkpoints).
void wave_program(SeisEngine* E, bool adjoint, bool ckmode, std::vector<WaveStage>& st, std::vector<WaveCopy>& cp)
{
    if (!ckmode) {
        if (adjoint) wave_steps_adj(E, st, 0, E->nt);
        else wave_steps_fwd(E, st, 0, E->nt);
        return;
    }
    const long long NP = E->g.NP;
    const int k = E->ck, L = k + 1, ncp = (E->nt + k - 1) / k;
    auto copy = [&](const float* src, long long ss, float* dst, long long ds) {
        st.push_back({kWaveCopy, 0, (int)cp.size(), 0});
        cp.push_back({src, dst, ss, ds});
    };
    if (!adjoint) {
        for (int c = 0; c < ncp; ++c) {
            const int t0 = c * k, t1 = std::min(t0 + k, E->nt);
            copy(E->d_p + (long long)((t0 + 1) % 3) * NP, 3 * NP, E->d_ckp + (long long)c * NP, (long long)ncp * NP);
            copy(E->d_ring + (long long)(t0 % L) * NP, (long long)L * NP, E->d_cku + (long long)c * NP,
                 (long long)ncp * NP);
            wave_steps_fwd(E, st, t0, t1);
        }
    } else {
        for (int c = ncp - 1; c >= 0; --c) {
            const int t0 = c * k, t1 = std::min(t0 + k, E->nt);
            copy(E->d_ckp + (long long)c * NP, (long long)ncp * NP, E->d_p + (long long)((t0 + 1) % 3) * NP, 3 * NP);
            copy(E->d_cku + (long long)c * NP, (long long)ncp * NP, E->d_ring + (long long)(t0 % L) * NP,
                 (long long)L * NP);
            wave_steps_fwd(E, st, t0, t1);
            wave_steps_adj(E, st, t0, t1);
        }
    }
}

// Appends the groups of one engine's sweep over its first `active` slots (mode 0
// forward, 1 forward + tangent, 2 reverse) to `out` and its arguments to `args`, and
// zeroes their progress counters on `st`.  Items are numbered by wave_launch.
int wave_groups(SeisEngine* E, int mode, bool hist, bool ckmode, int active, int resident, std::vector<WaveGroup>& out,
                std::vector<WaveArgs>& args, cudaStream_t st)
{
    std::vector<WaveStage> stv;
    std::vector<WaveCopy> cpv;
    wave_program(E, mode == 2, ckmode, stv, cpv);
    std::string bytes(reinterpret_cast<const char*>(stv.data()), stv.size() * sizeof(WaveStage));
    bytes.append(reinterpret_cast<const char*>(cpv.data()), cpv.size() * sizeof(WaveCopy));
    int rc = 0;
    const char* dprog = static_cast<const char*>(wave_blob(E, bytes, st, &rc));
    if (rc) return rc;
    const int tiles = E->tiles_x * E->tiles_z;
    if ((rc = dalloc(E, &E->d_wave_progress, (size_t)E->slots * tiles)) != 0) return rc;
    CK(cudaMemsetAsync(E->d_wave_progress, 0, sizeof(int) * (size_t)active * tiles, st));
    const long long NP = E->g.NP;
    const int L = E->ck + 1;
    WaveArgs wa{};
    wa.f = ckmode ? make_fwd_args(E, mode == 1, false, E->d_ring, L) : make_fwd_args(E, mode == 1, hist);
    wa.a = make_adj_args(E);
    if (ckmode) {
        wa.a.u = E->d_ring;
        wa.a.ulevels = L;
        wa.a.u_slot_stride = (long long)L * NP;
    }
    WaveGroup G{};
    G.prog = reinterpret_cast<const WaveStage*>(dprog);
    G.copies = reinterpret_cast<const WaveCopy*>(dprog + stv.size() * sizeof(WaveStage));
    G.err = E->d_err;
    G.nstages = (int)stv.size();
    G.tiles_x = E->tiles_x;
    G.tiles_z = E->tiles_z;
    G.reach = (E->g.NX - (E->tiles_x - 1) * kTX < 4 || E->g.NZ - (E->tiles_z - 1) * kTZ < 4) ? 2 : 1;
    G.args = (int)args.size();
    args.push_back(wa);
    // a group's stages advance together: a few slots of a large grid keep its fields in
    // L2, with items enough per stage to keep every resident block busy twice over
    int gs = E->wave_group_slots;
    if (gs <= 0) gs = std::max(1, (2 * resident + tiles - 1) / tiles);
    for (int s0 = 0; s0 < active; s0 += gs) {
        G.slot0 = s0;
        G.nslots = std::min(gs, active - s0);
        G.progress = E->d_wave_progress + (long long)s0 * tiles;
        out.push_back(G);
    }
    return 0;
}

// Launches over `groups` (engines' arguments `args`, at most kMaxWaveArgs per launch:
// more engines are split over several launches in stream order); the group tables and
// the launch state live with engine E.
template <int MODE>
int wave_launch_t(SeisEngine* E, std::vector<WaveGroup>& groups, const std::vector<WaveArgs>& args, cudaStream_t st)
{
    if (groups.empty()) return 0;
    int rc = wave_resident_t<MODE>(E);
    if (rc) return rc;
    if ((rc = dalloc(E, &E->d_wave_state, 2)) != 0) return rc;
    std::unique_ptr<WaveParams<MODE>> P(new WaveParams<MODE>());
    WaveKernel<MODE> k = wave_kernel<MODE>(E);
    size_t g0 = 0;
    while (g0 < groups.size()) {
        const int a0 = groups[g0].args;
        size_t g1 = g0;
        while (g1 < groups.size() && groups[g1].args < a0 + kMaxWaveArgs) ++g1;
        // longest programs first: their dependency chains start early, shorter groups fill in
        std::stable_sort(groups.begin() + g0, groups.begin() + g1,
                         [](const WaveGroup& x, const WaveGroup& y) { return x.nstages > y.nstages; });
        long long total = 0;
        for (size_t g = g0; g < g1; ++g) {
            groups[g].first = total;
            total += (long long)groups[g].nstages * groups[g].nslots * groups[g].tiles_x * groups[g].tiles_z;
            groups[g].args -= a0;
        }
        std::memset(static_cast<void*>(P.get()), 0, sizeof(WaveParams<MODE>));
        for (int i = 0; i < kMaxWaveArgs && a0 + i < (int)args.size(); ++i) {
            P->f[i] = args[a0 + i].f;
            if constexpr (MODE == 2) P->a[i] = args[a0 + i].a;
        }
        std::string bytes(reinterpret_cast<const char*>(groups.data() + g0), (g1 - g0) * sizeof(WaveGroup));
        const WaveGroup* dg = static_cast<const WaveGroup*>(wave_blob(E, bytes, st, &rc));
        if (rc) return rc;
        CK(cudaMemsetAsync(E->d_wave_state, 0, 2 * sizeof(unsigned long long), st));
        P->L.groups = dg;
        P->L.ngroups = (int)(g1 - g0);
        P->L.total = total;
        P->L.next = E->d_wave_state;
        P->L.abort = reinterpret_cast<int*>(E->d_wave_state + 1);
        const unsigned grid = (unsigned)std::min<long long>(wave_resident_of(E, MODE), total);
        if (grid > 0) {
            k<<<grid, dim3(kBX, kBZ), wave_smem<MODE>(), st>>>(*P);
            CK(cudaGetLastError());
            E->launches++;
        }
        g0 = g1;
    }
    return 0;
}

int wave_launch(SeisEngine* E, int mode, std::vector<WaveGroup>& groups, const std::vector<WaveArgs>& args,
                cudaStream_t st)
{
    return mode == 0 ? wave_launch_t<0>(E, groups, args, st)
                     : (mode == 1 ? wave_launch_t<1>(E, groups, args, st) : wave_launch_t<2>(E, groups, args, st));
}

// The wavefront sweep of one engine's chunk (its first `active` slots).
int wave_sweep(SeisEngine* E, int mode, bool hist, bool ckmode, int active, cudaStream_t st)
{
    int rc = wave_resident_mode(E, mode);
    if (rc) return rc;
    std::vector<WaveGroup> groups;
    std::vector<WaveArgs> args;
    rc = wave_groups(E, mode, hist, ckmode, active, wave_resident_of(E, mode), groups, args, st);
    if (rc) return rc;
    return wave_launch(E, mode, groups, args, st);
}

int next_event(SeisEngine* E, int* idx)
{
    if (*idx >= (int)E->ev_pool.size()) {
        cudaEvent_t ev;
        CK(cudaEventCreate(&ev));
        E->ev_pool.push_back(ev);
    }
    return 0;
}

}  // namespace

// Does a cluster kernel shape apply to this geometry, and with which bands?
void plan_cluster(SeisEngine* E, const ClusterShape& S, SeisEngine::ClusterPlan* P)
{
    const bool adjoint = S.adjoint;
    const int C = S.C, RPT = S.RPT, W = S.W;
    const int NZ = E->g.NZ, pitch = E->g.pitch;
    P->ok = false;
    P->shape = &S;
    P->C = C;
    P->W = W;
    if (pitch != S.sp || E->g.NX + 4 > S.sp) return;
    if (W == 2 && E->g.NX % 2) return;            // column pairs tile an even width only
    P->R = (NZ + C - 1) / C;
    // with column pairs, bands of whole strips (every strip of all but the last band is full)
    if (W == 2 && NZ - (C - 1) * ((P->R + RPT - 1) / RPT * RPT) >= 2) P->R = (P->R + RPT - 1) / RPT * RPT;
    if (NZ - (C - 1) * P->R < 2) return;          // every band needs two rows to push
    P->G = (P->R + RPT - 1) / RPT;
    if (P->G < 1 || P->G * (pitch / W) > S.threads) return;
    P->threads = P->G * (pitch / W);
    // three wavefield buffers (+ the forward's alpha, or the adjoint's alpha, 1-kappa and history ring; the
    // tensor-memory adjoint: a two-level history ring only) and the mbarriers
    const size_t bufs = adjoint ? (size_t)(3 * (P->R + 4) + (S.tmem ? 2 : 5) * P->R)
                                : (size_t)((S.tangent ? 6 : 3) * (P->R + 4) + (S.alpha_smem ? P->R : 0) +
                                           (S.tangent && !S.tmem ? P->R : 0));
    P->smem = bufs * pitch * sizeof(float) +
              (adjoint ? 7 * sizeof(uint64_t) + (S.tmem ? sizeof(float) * (size_t)P->R : 0)
                       : 3 * sizeof(uint64_t) + sizeof(float) * E->nt * (S.tangent ? 2 : 1) +
                             sizeof(int) * (3 * (size_t)E->nrec + 1) + (S.tmem ? 8 : 0) +
                             (S.tmem && S.tangent ? 2 * sizeof(float) * (size_t)P->R : 0));
    if (P->smem > kSmemLimit) return;
    if (!adjoint) {
        P->ok = true;
        return;
    }
    // adjoint seeds: at most two receivers per thread (one column of one strip of RPT rows)
    std::vector<long long> keys;
    for (int r = 0; r < E->nrec; ++r) {
        const int k = E->rec_z[r] / P->R, rz = E->rec_z[r] - k * P->R;
        keys.push_back(((long long)k * P->G + rz / RPT) * pitch + E->rec_x[r] / W);
    }
    std::sort(keys.begin(), keys.end());
    for (size_t i = 0, run = 1; i < keys.size(); ++i, ++run) {
        if (i + 1 < keys.size() && keys[i + 1] == keys[i]) continue;
        if (run > 2) return;
        run = 0;
    }
    P->ok = true;
}

// The plan of a sweep in use: among the shapes that apply (plain forward: with
// the chosen cluster size), one with the preferred columns per thread if any.
const SeisEngine::ClusterPlan* active_plan(const SeisEngine* E, bool adjoint, bool tangent = false)
{
    const SeisEngine::ClusterPlan* best = nullptr;
    int best_score = -1;
    for (const SeisEngine::ClusterPlan& P : E->plans) {
        if (!P.ok || P.shape->adjoint != adjoint || P.shape->tangent != tangent ||
            (!adjoint && !tangent && E->fwd_cluster && P.C != E->fwd_cluster))
            continue;
        if (P.shape->shuffle && !(E->shuffle && !adjoint && !tangent)) continue;
        if (adjoint && E->adj_cluster && P.C != E->adj_cluster) continue;
        if (P.shape->tmem && adjoint && P.shape->RPT != (E->adj_rows ? E->adj_rows : 8)) continue;
        if (P.shape->tmem && !adjoint && !E->fwd_tmem) continue;
        // preferred columns per thread first; then the shape whose clusters cover the most SMs with this
        // engine's chunk of shots (10-CTA clusters for large chunks, 16-CTA ones for a few shots, which
        // each finish sooner); then the forward's neighbour access and tensor-memory variant
        const int cover = tangent ? 0 : std::min(E->slots, std::max(1, P.nclusters)) * P.C;
        const int score = 1000000 * (P.W == E->cols) + 4 * cover + 2 * (P.shape->shuffle == (E->shuffle != 0)) +
                          (!adjoint && P.shape->tmem == (E->fwd_tmem != 0));
        if (score > best_score) {
            best = &P;
            best_score = score;
        }
    }
    return best;
}
// Number of resident clusters of the first applicable shape with this sweep and cluster size (0: none).
int64_t plan_clusters(const SeisEngine* E, bool adjoint, int C, bool tangent = false)
{
    for (const SeisEngine::ClusterPlan& P : E->plans)
        if (P.ok && P.shape->adjoint == adjoint && P.shape->tangent == tangent && P.C == C) return P.nclusters;
    return 0;
}

template <class K>
int cluster_occupancy(SeisEngine* E, K kernel, SeisEngine::ClusterPlan* P)
{
    // the attribute belongs to the kernel, not to this engine: allow the opt-in
    // maximum so that every engine's launch (each with its own size) stays valid
    cudaFuncAttributes fa{};
    CK(cudaFuncGetAttributes(&fa, kernel));
    const size_t dyn_max = kSmemLimit - fa.sharedSizeBytes;   // static + dynamic <= the opt-in limit
    if (P->smem > dyn_max) { P->ok = false; return 0; }
    CK(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn_max));
    if (P->C > 8) CK(cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = P->C;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(P->C, 1, 1);
    cfg.blockDim = dim3(P->threads, 1, 1);
    cfg.dynamicSmemBytes = P->smem;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int n = 0;
    CK(cudaOccupancyMaxActiveClusters(&n, (void*)kernel, &cfg));
    P->nclusters = n;
    if (n < 1) P->ok = false;
    return 0;
}

template <class K>
int launch_cluster(SeisEngine* E, K kernel, const SeisEngine::ClusterPlan& P, int active, const ClusterArgs& a,
                   cudaStream_t st)
{
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = P.C;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    const int ncl = std::max(1, std::min(P.nclusters, active));
    cfg.gridDim = dim3(P.C * ncl, 1, 1);
    cfg.blockDim = dim3(P.threads, 1, 1);
    cfg.dynamicSmemBytes = P.smem;
    cfg.stream = st;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    CK(cudaLaunchKernelEx(&cfg, kernel, a));
    return 0;
}

ClusterArgs make_cluster_args(SeisEngine* E, const SeisEngine::ClusterPlan& P, bool hist)
{
    ClusterArgs a{};
    a.g = E->g;
    a.R = P.R;
    a.G = P.G;
    a.slots = E->slots;
    a.shots = E->d_shots;
    a.alpha = E->d_alpha;
    a.kfac = E->d_kfac;
    a.dampx = E->d_dampx;
    a.dampz = E->d_dampz;
    a.rec_z = E->d_rec_z;
    a.rec_x = E->d_rec_x;
    a.smod = E->d_smod;
    a.rec = E->d_rec;
    a.alpha_d = E->d_alpha_d;
    a.kdfac = E->d_kdfac;
    a.smod_d = E->d_smod_d;
    a.drec = E->d_drec;
    a.uhist = hist ? E->d_uhist : nullptr;
    a.u_slot_stride = (long long)(E->nt + 1) * E->g.NP;
    a.write_hist = hist ? 1 : 0;
    a.seed = E->d_seed;
    a.gv = E->d_gv;
    a.gk = E->d_gk;
    a.err = E->d_err;
    a.skip_copy_level = E->skip_copy_level;
    return a;
}

// The cluster shape of the forward side slots (option fwd_side_cluster), or none.
// Automatic: 8-CTA clusters beside a 10-CTA main forward that leaves at least two
// clusters' worth of SMs free (on GB300 two 8-CTA clusters run on the 22 SMs that 13
// ten-CTA clusters leave, measured; a third does not fit).
const SeisEngine::ClusterPlan* side_cluster_plan(const SeisEngine* E, bool tangent)
{
    if (!E->fwd_side_cluster || tangent) return nullptr;
    int C = E->fwd_side_cluster;
    if (C < 0) {
        const SeisEngine::ClusterPlan* fp = active_plan(E, false);
        if (!fp || fp->C != 10 || E->num_sms - fp->nclusters * fp->C < 8 * E->fwd_side_clusters) return nullptr;
        C = 8;
    }
    for (const SeisEngine::ClusterPlan& P : E->plans)
        if (P.ok && !P.shape->adjoint && !P.shape->tangent && !P.shape->tmem && !P.shape->shuffle && P.C == C &&
            P.W == E->cols)
            return &P;
    return nullptr;
}

// Forward side slots on cluster sweeps: the main clusters take r whole rounds (r * ncl
// slots), the k side clusters the rest; r minimises max(r, ceil(side / k) * rho) where rho
// is a side cluster's time per shot in main rounds.  option >= 0: exactly that many.
void side_split_clusters(const SeisEngine::ClusterPlan& P, int S, int option, int k, double rho, int* s0, int* ns)
{
    int side = option;
    if (option < 0) {
        const int ncl = std::max(1, P.nclusters);
        double best = 1e30;
        side = 0;
        for (int r = 1; r <= (S + ncl - 1) / ncl; ++r) {
            const int sd = std::max(0, S - r * ncl);
            const double t = std::max((double)r, std::ceil((double)sd / k) * rho);
            if (t < best) {
                best = t;
                side = sd;
            }
        }
    }
    *s0 = S;
    *ns = 0;
    if (side > 0 && side < S) {
        *s0 = S - side;
        *ns = side;
    }
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------

extern "C" const char* seis_last_error(const SeisEngine* engine)
{
    return engine ? engine->err.c_str() : g_create_error.c_str();
}

extern "C" int seis_create(const SeisGeometry* G, int32_t max_models, int32_t max_shots_per_chunk,
                           SeisEngine** out)
{
    g_create_error.clear();
    auto bad = [](const char* m) { g_create_error = m; return SEIS_E_INVALID; };
    if (!G || !out) return bad("seis_create: null geometry or output pointer");
    *out = nullptr;
    if (G->nz < 1 || G->nx < 1) return bad("seis_create: nz and nx must be >= 1");
    if (G->nbc < 2) return bad("seis_create: nbc must be >= 2");
    if (G->nt < 1) return bad("seis_create: nt must be >= 1");
    if (!(G->dx > 0) || !(G->dt > 0) || !(G->freq > 0)) return bad("seis_create: dx, dt and freq must be > 0");
    if (G->nshots < 1 || !G->src_z || !G->src_x) return bad("seis_create: need >= 1 shot with positions");
    if (G->nrec < 1 || !G->rec_z || !G->rec_x) return bad("seis_create: need >= 1 receiver with positions");
    if (max_models < 1) return bad("seis_create: max_models must be >= 1");
    if (max_shots_per_chunk < 0) return bad("seis_create: max_shots_per_chunk must be >= 0");
    const int NZ = G->nz + 2 * G->nbc, NX = G->nx + 2 * G->nbc;
    if ((long long)NZ * NX > (1LL << 30)) return bad("seis_create: padded grid too large");
    for (int s = 0; s < G->nshots; ++s)
        if (G->src_z[s] < 0 || G->src_z[s] >= NZ || G->src_x[s] < 0 || G->src_x[s] >= NX)
            return bad("seis_create: source outside the padded grid");
    for (int r = 0; r < G->nrec; ++r)
        if (G->rec_z[r] < 0 || G->rec_z[r] >= NZ || G->rec_x[r] < 0 || G->rec_x[r] >= NX)
            return bad("seis_create: receiver outside the padded grid");
    std::vector<double> ricker;
    if (host_ricker(G->freq, G->dt, G->nt, ricker) < 0) return bad("seis_create: nt is smaller than the Ricker wavelet");

    SeisEngine* E = new SeisEngine();
    E->nz = G->nz; E->nx = G->nx; E->nbc = G->nbc; E->nt = G->nt;
    E->dx = G->dx; E->dt = G->dt; E->freq = G->freq;
    E->nshots = G->nshots; E->nrec = G->nrec;
    E->src_z.assign(G->src_z, G->src_z + G->nshots);
    E->src_x.assign(G->src_x, G->src_x + G->nshots);
    E->rec_z.assign(G->rec_z, G->rec_z + G->nrec);
    E->rec_x.assign(G->rec_x, G->rec_x + G->nrec);
    const int pitch = (NX + 31) / 32 * 32;
    E->g.NZ = NZ; E->g.NX = NX; E->g.pitch = pitch;
    E->g.xlo = G->nbc; E->g.xhi = G->nbc + G->nx;
    E->g.NP = (long long)NZ * pitch;
    E->g.nt = G->nt; E->g.nrec = G->nrec;
    E->mg = ModelGeom{G->nz, G->nx, G->nbc, G->dt, G->dx};
    E->tiles_x = (NX + kTX - 1) / kTX;
    E->tiles_z = (NZ + kTZ - 1) / kTZ;
    E->max_models = max_models;
    const int total_shots = max_models * G->nshots;
    int slots = max_shots_per_chunk;
    if (slots <= 0) {
        // default: as many concurrently swept shots as 60% of free device memory holds
        // with a gradient workspace (the history dominates: (nt+1) levels per shot)
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) free_b = (size_t)16 << 30;
        const double per_slot = 4.0 * (double)(G->nt + 15) * (double)E->g.NP;
        slots = (int)std::max(1.0, std::min(4096.0, 0.6 * (double)free_b / per_slot));
    }
    E->slots = std::max(1, std::min(slots, total_shots));

    auto fail_create = [&](int code) {
        g_create_error = E->err;
        free_all(E);
        delete E;
        return code;
    };
    int rc = 0;
#define CR(x) do { if ((rc = (x)) != 0) return fail_create(rc); } while (0)
    // constants
    std::vector<double> dx64, dz64;
    host_damp_profiles(G->nbc, G->nz, G->nx, G->dx, pitch, NZ, dx64, dz64);
    std::vector<float> dx32(dx64.begin(), dx64.end()), dz32(dz64.begin(), dz64.end());
    std::vector<int> rec_off(G->nrec);
    for (int r = 0; r < G->nrec; ++r) rec_off[r] = G->rec_z[r] * pitch + G->rec_x[r];
    const int ntiles = E->tiles_x * E->tiles_z;
    std::vector<int> tstart(ntiles + 1, 0), tlist;
    {
        std::vector<std::vector<int>> per(ntiles);
        for (int r = 0; r < G->nrec; ++r)
            per[(G->rec_z[r] / kTZ) * E->tiles_x + G->rec_x[r] / kTX].push_back(r);
        for (int t = 0; t < ntiles; ++t) {
            tstart[t] = (int)tlist.size();
            tlist.insert(tlist.end(), per[t].begin(), per[t].end());
        }
        tstart[ntiles] = (int)tlist.size();
    }
    auto up = [&](auto** dst, const auto* src, size_t n) -> int {
        CR(dalloc(E, dst, n));
        cudaError_t e = cudaMemcpy(*dst, src, sizeof(**dst) * n, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return E->fail(SEIS_E_CUDA, "cudaMemcpy (constants) failed: %s", cudaGetErrorString(e));
        return 0;
    };
    CR(up(&E->d_dampx, dx32.data(), dx32.size()));
    CR(up(&E->d_dampz, dz32.data(), dz32.size()));
    CR(up(&E->d_dampx64, dx64.data(), dx64.size()));
    CR(up(&E->d_dampz64, dz64.data(), dz64.size()));
    CR(up(&E->d_ricker, ricker.data(), ricker.size()));
    CR(up(&E->d_src_z, E->src_z.data(), E->src_z.size()));
    CR(up(&E->d_src_x, E->src_x.data(), E->src_x.size()));
    CR(up(&E->d_rec_off, rec_off.data(), rec_off.size()));
    CR(up(&E->d_tile_rec_start, tstart.data(), tstart.size()));
    CR(up(&E->d_tile_rec_list, tlist.data(), std::max<size_t>(1, tlist.size())));
    CR(up(&E->d_rec_z, E->rec_z.data(), E->rec_z.size()));
    CR(up(&E->d_rec_x, E->rec_x.data(), E->rec_x.size()));
    CR(dalloc(E, &E->d_err, 1));
    {
        cudaError_t e = cudaMemset(E->d_err, 0, sizeof(int));
        if (e == cudaSuccess) e = cudaHostAlloc((void**)&E->h_err, sizeof(int), cudaHostAllocDefault);
        if (e != cudaSuccess) {
            E->fail(SEIS_E_CUDA, "error word set-up failed: %s", cudaGetErrorString(e));
            return fail_create(SEIS_E_CUDA);
        }
        *E->h_err = 0;
    }
    for (int i = 0; i < kNumShapes; ++i) {
        plan_cluster(E, kShapes[i], &E->plans[i]);
        if (E->plans[i].ok) CR(cluster_occupancy(E, kShapes[i].kernel, &E->plans[i]));
    }
    {
        // the two-step tiled adjoint's and tangent's shared memory is above the 48 KB default
        cudaError_t e = cudaSuccess;
        for (auto k : {adj_step2_kernel<1>, adj_step2_kernel<2>, adj_step2_kernel<4>})
            if (e == cudaSuccess) e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, kFusedAdjSmem);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(fwd_step2_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     fused_fwd_smem<true>());
        if (e != cudaSuccess) {
            E->fail(SEIS_E_CUDA, "cudaFuncSetAttribute (two-step tiled sweeps) failed: %s", cudaGetErrorString(e));
            return fail_create(SEIS_E_CUDA);
        }
    }
    {
        cudaError_t e = cudaStreamCreateWithFlags(&E->cap_stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&E->io_stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&E->io_ev, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&E->io_in_ev, cudaEventDisableTiming);
        int lo_prio = 0, hi_prio = 0;
        if (e == cudaSuccess) e = cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio);
        int dev = 0;
        if (e == cudaSuccess) e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&E->num_sms, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&E->hi_stream, cudaStreamNonBlocking, hi_prio);
        if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&E->side_stream, cudaStreamNonBlocking, lo_prio);
        for (cudaEvent_t* ev : {&E->fork_ev, &E->join_hi_ev, &E->join_side_ev})
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
        if (e != cudaSuccess) {
            E->fail(SEIS_E_CUDA, "cudaStreamCreateWithFlags failed: %s", cudaGetErrorString(e));
            return fail_create(SEIS_E_CUDA);
        }
    }
#undef CR
    *out = E;
    return 0;
}

extern "C" int seis_chunk_slots(const SeisEngine* E) { return E ? E->slots : SEIS_E_INVALID; }

extern "C" int seis_set_option(SeisEngine* E, const char* key, int64_t value)
{
    if (!E || !key) return SEIS_E_INVALID;
    std::lock_guard<std::mutex> lk(E->mu);
    if (!strcmp(key, "sweep_path")) {
        if (value < 0 || value > 3) return E->fail(SEIS_E_INVALID, "sweep_path must be 0, 1, 2 or 3");
        if (value == 2 && !(plan_clusters(E, false, 8) + plan_clusters(E, false, 10) + plan_clusters(E, false, 16) > 0 &&
                            plan_clusters(E, true, 16) > 0))
            return E->fail(SEIS_E_INVALID, "cluster sweeps do not apply to this geometry");
        E->path = (int)value;
        return 0;
    }
    if (!strcmp(key, "fwd_cluster")) {
        if (value != 0 && value != 8 && value != 10 && value != 16)
            return E->fail(SEIS_E_INVALID, "fwd_cluster must be 0, 8, 10 or 16");
        if (value && value != 8 && !plan_clusters(E, false, (int)value))
            return E->fail(SEIS_E_INVALID, "%d-CTA forward clusters do not apply", (int)value);
        E->fwd_cluster = (int)value;
        return 0;
    }
    if (!strcmp(key, "adj_cluster")) {
        if (value != 0 && value != 10 && value != 16) return E->fail(SEIS_E_INVALID, "adj_cluster must be 0, 10 or 16");
        if (value && !plan_clusters(E, true, (int)value))
            return E->fail(SEIS_E_INVALID, "%d-CTA adjoint clusters do not apply", (int)value);
        E->adj_cluster = (int)value;
        return 0;
    }
    if (!strcmp(key, "fwd_tmem")) {
        if (value != 0 && value != 1) return E->fail(SEIS_E_INVALID, "fwd_tmem must be 0 or 1");
        E->fwd_tmem = (int)value;
        return 0;
    }
    if (!strcmp(key, "adj_rows")) {
        if (value != 0 && value != 8 && value != 11) return E->fail(SEIS_E_INVALID, "adj_rows must be 0, 8 or 11");
        E->adj_rows = (int)value;
        return 0;
    }
    if (!strcmp(key, "neighbour_shuffle")) {
        if (value != 0 && value != 1) return E->fail(SEIS_E_INVALID, "neighbour_shuffle must be 0 or 1");
        E->shuffle = (int)value;
        return 0;
    }
    if (!strcmp(key, "columns")) {
        if (value != 1 && value != 2) return E->fail(SEIS_E_INVALID, "columns must be 1 or 2");
        E->cols = (int)value;
        return 0;
    }
    if (!strcmp(key, "test_skip_history_copy")) {
        // never issue the adjoint's history copy of this level: its bounded wait runs
        // out (about 2 s), the sweep reports SEIS_E_TIMEOUT through seis_device_status
        // and the results of that call are invalid; -1 turns it off
        if (value < -1 || value > E->nt) return E->fail(SEIS_E_INVALID, "test_skip_history_copy out of range");
        E->skip_copy_level = (int)value;
        return 0;
    }
    if (!strcmp(key, "adj_fuse") || !strcmp(key, "adj_hoist")) {
        const bool fuse = !strcmp(key, "adj_fuse");
        if (fuse ? (value != 0 && value != 1) : (value != 1 && value != 2 && value != 4))
            return E->fail(SEIS_E_INVALID, fuse ? "adj_fuse must be 0 or 1" : "adj_hoist must be 1, 2 or 4");
        int& field = fuse ? E->adj_fuse : E->adj_hoist;
        if (field != (int)value) {
            field = (int)value;
            if (E->adj_graph) { cudaGraphExecDestroy(E->adj_graph); E->adj_graph = nullptr; }
            if (E->ck_adj_graph) { cudaGraphExecDestroy(E->ck_adj_graph); E->ck_adj_graph = nullptr; }
            destroy_graphs(E->adj_side_graphs);
        }
        return 0;
    }
    if (!strcmp(key, "adj_side") || !strcmp(key, "fwd_side")) {
        if (value < -1 || value >= E->slots) return E->fail(SEIS_E_INVALID, "%s must be in [-1, slots)", key);
        (key[0] == 'a' ? E->adj_side : E->fwd_side) = (int)value;
        return 0;
    }
    if (!strcmp(key, "fwd_side_cluster")) {
        if (value != -1 && value != 0 && value != 8 && value != 10 && value != 16)
            return E->fail(SEIS_E_INVALID, "fwd_side_cluster must be -1, 0, 8, 10 or 16");
        E->fwd_side_cluster = (int)value;
        return 0;
    }
    if (!strcmp(key, "fwd_side_clusters")) {
        if (value < 1 || value > 16) return E->fail(SEIS_E_INVALID, "fwd_side_clusters must be in [1, 16]");
        E->fwd_side_clusters = (int)value;
        return 0;
    }
    if (!strcmp(key, "fwd_fuse")) {
        if (value != 0 && value != 1) return E->fail(SEIS_E_INVALID, "fwd_fuse must be 0 or 1");
        if (E->fwd_fuse != (int)value) {
            E->fwd_fuse = (int)value;
            for (auto& row : E->fwd_graph)
                for (auto& gexec : row)
                    if (gexec) { cudaGraphExecDestroy(gexec); gexec = nullptr; }
            for (auto& gexec : E->ck_fwd_graph)
                if (gexec) { cudaGraphExecDestroy(gexec); gexec = nullptr; }
            for (auto& row : E->fwd_side_graphs)
                for (auto& v : row) destroy_graphs(v);
            if (E->ck_adj_graph) { cudaGraphExecDestroy(E->ck_adj_graph); E->ck_adj_graph = nullptr; }
        }
        return 0;
    }
    if (!strcmp(key, "wave_fwd_blocks")) {
        if (value < 4 || value > 6) return E->fail(SEIS_E_INVALID, "wave_fwd_blocks must be 4, 5 or 6");
        E->wave_fwd_blocks = (int)value;
        return 0;
    }
    if (!strcmp(key, "wave_group_slots")) {
        if (value < 0) return E->fail(SEIS_E_INVALID, "wave_group_slots must be >= 0");
        E->wave_group_slots = (int)value;
        return 0;
    }
    if (!strcmp(key, "checkpoint_every")) {
        if (value < 0 || value > E->nt) return E->fail(SEIS_E_INVALID, "checkpoint_every must be in [0, nt]");
        E->ck = (int)value;
        return 0;
    }
    return E->fail(SEIS_E_INVALID, "unknown option '%s'", key);
}

extern "C" int seis_get_info(const SeisEngine* E, const char* key, int64_t* value)
{
    if (!E || !key || !value) return SEIS_E_INVALID;
    SeisEngine* M = const_cast<SeisEngine*>(E);
    std::lock_guard<std::mutex> lk(M->mu);
    const SeisEngine::ClusterPlan* fp = active_plan(E, false);
    const SeisEngine::ClusterPlan* ap = active_plan(E, true);
    if (!strcmp(key, "cluster_fwd")) *value = plan_clusters(E, false, 8);
    else if (!strcmp(key, "fwd_columns")) *value = fp ? fp->W : 0;
    else if (!strcmp(key, "fwd_shuffle")) *value = fp ? (int64_t)fp->shape->shuffle : 0;
    else if (!strcmp(key, "fwd_tmem")) *value = fp ? (int64_t)fp->shape->tmem : 0;
    else if (!strcmp(key, "adj_columns")) *value = ap ? ap->W : 0;
    else if (!strcmp(key, "cluster_adj")) *value = ap ? ap->nclusters : 0;
    else if (!strcmp(key, "adj_cluster")) *value = ap ? ap->C : 0;
    else if (!strcmp(key, "adj_tmem")) *value = ap ? (int64_t)ap->shape->tmem : 0;
    else if (!strcmp(key, "cluster_tan")) *value = plan_clusters(E, false, 16, true);
    else if (!strcmp(key, "sweep_path")) *value = E->path;
    else if (!strcmp(key, "checkpoint_every")) *value = E->ck;
    else if (!strcmp(key, "adj_hoist")) *value = E->adj_hoist;
    else if (!strcmp(key, "fwd_cluster")) *value = fp ? fp->C : E->fwd_cluster;
    else if (!strcmp(key, "cluster_fwd16"))
        *value = plan_clusters(E, false, 16);
    else if (!strcmp(key, "cluster_fwd10"))
        *value = plan_clusters(E, false, 10);
    else if (!strcmp(key, "slots")) *value = E->slots;
    else if (!strcmp(key, "tiles")) *value = (int64_t)E->tiles_x * E->tiles_z;
    else if (!strcmp(key, "last_fwd_launches")) *value = E->last_fwd_launches;
    else if (!strcmp(key, "last_adj_launches")) *value = E->last_adj_launches;
    else if (!strcmp(key, "last_fwd_path")) *value = E->last_fwd_path;
    else if (!strcmp(key, "last_adj_path")) *value = E->last_adj_path;
    else if (!strcmp(key, "last_adj_side")) *value = E->last_adj_side;
    else if (!strcmp(key, "last_adj_cluster_ns")) {
        // device time of the last call's cluster adjoint launches, one per chunk (beside
        // the side adjoint where a chunk has one); the call's stream must have been
        // synchronised
        double ns = 0.0;
        if (E->last_adj_path == 2)
            for (const auto& pr : M->adj_cl_ev) {
                float ms = 0.0f;
                cudaError_t e = cudaEventElapsedTime(&ms, M->ev_pool[pr.first], M->ev_pool[pr.second]);
                if (e != cudaSuccess)
                    return M->fail(SEIS_E_CUDA, "last_adj_cluster_ns: %s", cudaGetErrorString(e));
                ns += 1e6 * (double)ms;
            }
        *value = (int64_t)ns;
    }
    else if (!strcmp(key, "adj_side")) *value = E->adj_side;
    else if (!strcmp(key, "fwd_side")) *value = E->fwd_side;
    else if (!strcmp(key, "last_fwd_side")) *value = E->last_fwd_side;
    else if (!strcmp(key, "fwd_side_cluster")) {
        const SeisEngine::ClusterPlan* sp = side_cluster_plan(E, false);
        *value = sp ? sp->C : 0;
    }
    else if (!strcmp(key, "wave_group_slots")) *value = E->wave_group_slots;
    else if (!strcmp(key, "err_word")) *value = *E->h_err;   // no sync: valid once the call's stream is done
    else return M->fail(SEIS_E_INVALID, "unknown info key '%s'", key);
    return 0;
}

extern "C" int seis_device_status(SeisEngine* E)
{
    if (!E) return SEIS_E_INVALID;
    std::lock_guard<std::mutex> lk(E->mu);
    CK(cudaStreamSynchronize(E->last_stream));
    int h = 0;
    CK(cudaMemcpy(&h, E->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (h) {
        // reported once: clear the sticky word so that later calls start clean
        CK(cudaMemset(E->d_err, 0, sizeof(int)));
        *E->h_err = 0;
        return E->fail(SEIS_E_TIMEOUT,
                       "a sweep gave up a bounded wait since the last status check (error word %d: 1 "
                       "history copy, 2 copy pending at exit, 4 halo rows, 8 wavefront tile); the results of that "
                       "call are invalid",
                       h);
    }
    return 0;
}

extern "C" int seis_destroy(SeisEngine* E)
{
    if (!E) return SEIS_E_INVALID;
    {
        std::lock_guard<std::mutex> lk(E->mu);
        free_all(E);
    }
    delete E;
    return 0;
}

static int vel_to_seis_call(SeisEngine* E, int32_t nmodels, const double* vec, const double* vec_diff,
                            const double* vec_adjoint, int32_t on_residual, double* result, double* result_diff,
                            double* result_adjoint, double* misfit, void* stream, bool gn);

namespace {

// Host memory (pinned or pageable) rather than device memory?  A pointer the
// runtime does not recognise is left to the device path, as before.
bool host_ptr(const void* p)
{
    if (!p) return false;
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeHost || at.type == cudaMemoryTypeUnregistered;
}

// A call whose inputs or outputs may live in host memory.  Host inputs are
// uploaded into device staging: vec and vec_diff on the call's stream, vec_adjoint
// on the engine's copy stream while the forward sweep runs (the seeds wait for
// it).  Host records go down chunk by chunk on the copy stream while the adjoint
// sweep runs; the gradient and misfit at the end.  The call's stream waits for
// the copy stream before the call returns, so stream order covers every copy.
int staged_call(SeisEngine* E, int32_t nmodels, const double* vec, const double* vec_diff, const double* vec_adjoint,
                int32_t on_residual, double* result, double* result_diff, double* result_adjoint, double* misfit,
                void* stream, bool gn)
{
    const bool hv = host_ptr(vec), hvd = host_ptr(vec_diff), hva = host_ptr(vec_adjoint);
    const bool hr = host_ptr(result), hrd = host_ptr(result_diff), hra = host_ptr(result_adjoint),
               hmf = host_ptr(misfit);
    if (!(hv || hvd || hva || hr || hrd || hra || hmf))
        return vel_to_seis_call(E, nmodels, vec, vec_diff, vec_adjoint, on_residual, result, result_diff,
                                result_adjoint, misfit, stream, gn);
    E->err.clear();
    if (nmodels < 1 || nmodels > E->max_models)
        return E->fail(SEIS_E_INVALID, "nmodels=%d outside [1, %d]", nmodels, E->max_models);
    cudaStream_t st = (cudaStream_t)stream;
    const size_t M = (size_t)E->max_models, nv = (size_t)E->nz * E->nx + 1;
    const size_t nrecords = (size_t)E->nshots * E->nt * E->nrec;
    const size_t m = (size_t)nmodels;
    int rc = 0;
#define CA(x) do { if ((rc = (x)) != 0) return rc; } while (0)
    if (hv) CA(dalloc(E, &E->d_in_vec, M * nv));
    if (hvd) CA(dalloc(E, &E->d_in_vd, M * nv));
    if (hva) CA(dalloc(E, &E->d_in_va, M * nrecords));
    if (hr) CA(dalloc(E, &E->d_out_res, M * nrecords));
    if (hrd) CA(dalloc(E, &E->d_out_rd, M * nrecords));
    if (hra) CA(dalloc(E, &E->d_out_ra, M * nv));
    if (hmf) CA(dalloc(E, &E->d_out_mf, M));
#undef CA
    // the copy stream starts after everything before this call on the call's stream
    CK(cudaEventRecord(E->io_ev, st));
    CK(cudaStreamWaitEvent(E->io_stream, E->io_ev, 0));
    if (hv) {
        CK(cudaMemcpyAsync(E->d_in_vec, vec, sizeof(double) * m * nv, cudaMemcpyHostToDevice, st));
        vec = E->d_in_vec;
    }
    if (hvd) {
        CK(cudaMemcpyAsync(E->d_in_vd, vec_diff, sizeof(double) * m * nv, cudaMemcpyHostToDevice, st));
        vec_diff = E->d_in_vd;
    }
    if (hva) {
        CK(cudaMemcpyAsync(E->d_in_va, vec_adjoint, sizeof(double) * m * nrecords, cudaMemcpyHostToDevice,
                           E->io_stream));
        CK(cudaEventRecord(E->io_in_ev, E->io_stream));
        vec_adjoint = E->d_in_va;
    }
    E->io.wait_va = hva;
    E->io.res = hr ? result : nullptr;
    E->io.rd = hrd ? result_diff : nullptr;
    double* res_d = hr ? E->d_out_res : result;
    double* rd_d = hrd ? E->d_out_rd : result_diff;
    double* ra_d = hra ? E->d_out_ra : result_adjoint;
    double* mf_d = hmf ? E->d_out_mf : misfit;
    rc = vel_to_seis_call(E, nmodels, vec, vec_diff, vec_adjoint, on_residual, res_d, rd_d, ra_d, mf_d, stream, gn);
    E->io = SeisEngine::HostIO{};
    // join the copy stream back into the call's stream, then the end-of-call results
    CK(cudaEventRecord(E->io_ev, E->io_stream));
    CK(cudaStreamWaitEvent(st, E->io_ev, 0));
    if (rc) return rc;
    if (hra) CK(cudaMemcpyAsync(result_adjoint, ra_d, sizeof(double) * m * nv, cudaMemcpyDeviceToHost, st));
    if (hmf) CK(cudaMemcpyAsync(misfit, mf_d, sizeof(double) * m, cudaMemcpyDeviceToHost, st));
    return 0;
}

}  // namespace

extern "C" int seis_vel_to_seis(SeisEngine* E, int32_t nmodels, const double* vec, const double* vec_diff,
                                const double* vec_adjoint, int32_t on_residual, double* result,
                                double* result_diff, double* result_adjoint, double* misfit, void* stream)
{
    if (!E) return SEIS_E_INVALID;
    std::lock_guard<std::mutex> lk(E->mu);
    return staged_call(E, nmodels, vec, vec_diff, vec_adjoint, on_residual, result, result_diff, result_adjoint,
                       misfit, stream, false);
}

extern "C" int seis_gn_matvec(SeisEngine* E, int32_t nmodels, const double* vec, const double* vec_diff,
                              double* result, double* result_diff, double* result_adjoint, void* stream)
{
    if (!E) return SEIS_E_INVALID;
    std::lock_guard<std::mutex> lk(E->mu);
    return staged_call(E, nmodels, vec, vec_diff, nullptr, 0, result, result_diff, result_adjoint, nullptr, stream,
                       true);
}

extern "C" int seis_stats(const SeisEngine* Ec, int64_t* launches, double* fwd_ms, double* adj_ms,
                          int64_t* fwd_step_launches, int64_t* adj_step_launches)
{
    if (!Ec) return SEIS_E_INVALID;
    SeisEngine* E = const_cast<SeisEngine*>(Ec);
    std::lock_guard<std::mutex> lk(E->mu);
    if (launches) *launches = E->launches;
    if (fwd_step_launches) *fwd_step_launches = E->fwd_step_launches;
    if (adj_step_launches) *adj_step_launches = E->adj_step_launches;
    auto total = [&](const std::vector<std::pair<int, int>>& v, double* o) -> int {
        double s = 0.0;
        for (auto& pr : v) {
            float ms = 0.0f;
            CK(cudaEventElapsedTime(&ms, E->ev_pool[pr.first], E->ev_pool[pr.second]));
            s += ms;
        }
        if (o) *o = s;
        return 0;
    };
    int rc = total(E->fwd_ev, fwd_ms);
    if (rc) return rc;
    return total(E->adj_ev, adj_ms);
}

// One call of the engine (the body of seis_vel_to_seis and seis_gn_matvec).
// gn: the adjoint's seeds are this call's own tangent records (J v), so one
// call returns J v and J^T J v; vec_adjoint is then unused.
namespace {

// Workspace of a call (allocated on first need, kept for the engine's lifetime).
int call_workspace(SeisEngine* E, bool tan, bool adj, bool ckmode)
{
    const long long NP = E->g.NP;
    const size_t S = (size_t)E->slots, M = (size_t)E->max_models;
    const long long per_shot = (long long)E->nt * E->nrec;
    int rc = 0;
#define CA(x) do { if ((rc = (x)) != 0) return rc; } while (0)
    CA(dalloc(E, &E->d_alpha, M * NP));
    CA(dalloc(E, &E->d_kfac, M));
    CA(dalloc(E, &E->d_shots, S));
    CA(dalloc(E, &E->d_p, S * 3 * NP));
    CA(dalloc(E, &E->d_smod, S * E->nt));
    CA(dalloc(E, &E->d_rec, S * per_shot));
    if (tan) {
        CA(dalloc(E, &E->d_alpha_d, M * NP));
        CA(dalloc(E, &E->d_kdfac, M));
        CA(dalloc(E, &E->d_dp, S * 3 * NP));
        CA(dalloc(E, &E->d_du, S * 3 * NP));
        CA(dalloc(E, &E->d_smod_d, S * E->nt));
        CA(dalloc(E, &E->d_drec, S * per_shot));
    }
    if (ckmode && E->ck_alloc_k != (size_t)E->ck) {
        dfree(E->d_ckp);
        dfree(E->d_cku);
        dfree(E->d_ring);
        const size_t ncp = (size_t)(E->nt + E->ck - 1) / E->ck;
        CA(dalloc(E, &E->d_ckp, S * ncp * NP));
        CA(dalloc(E, &E->d_cku, S * ncp * NP));
        CA(dalloc(E, &E->d_ring, S * (size_t)(E->ck + 1) * NP));
        E->ck_alloc_k = (size_t)E->ck;
    }
    if (adj) {
        if (!ckmode) CA(dalloc(E, &E->d_uhist, S * (size_t)(E->nt + 1) * NP));
        CA(dalloc(E, &E->d_lam, S * 3 * NP));
        CA(dalloc(E, &E->d_mu, S * 3 * NP));
        CA(dalloc(E, &E->d_gv, S * NP));
        CA(dalloc(E, &E->d_gk, S * NP));
        CA(dalloc(E, &E->d_seed, S * per_shot));
        CA(dalloc(E, &E->d_acc_v, M * std::max<size_t>((size_t)NP, kMisfitParts)));   // also the misfit's partial sums
        CA(dalloc(E, &E->d_acc_k, M * NP));
    } else {
        CA(dalloc(E, &E->d_uring, S * 3 * NP));
    }
#undef CA
    return 0;
}

// Chunk set-up: slots -> (model, shot) and their source terms, zero wavefields, level 0
// of u (u_1 = 0) of every active slot (the sweep writes every later level).
int chunk_begin(SeisEngine* E, int first, int total_shots, int active, const double* vec, const double* vec_diff,
                bool tan, float* ubuf, size_t ulevels, cudaStream_t st)
{
    const long long NP = E->g.NP;
    const size_t S = (size_t)E->slots;
    chunk_setup_kernel<<<(unsigned)S, 128, 0, st>>>(E->g, E->mg, first, total_shots, E->nshots, E->d_src_z,
                                                    E->d_src_x, vec, vec_diff, E->d_ricker, E->d_shots,
                                                    E->d_smod, E->d_smod_d);
    E->launches++;
    CK(cudaMemsetAsync(E->d_p, 0, sizeof(float) * S * 3 * NP, st));
    CK(cudaMemset2DAsync(ubuf, sizeof(float) * ulevels * NP, 0, sizeof(float) * NP, (size_t)active, st));
    if (tan) {
        CK(cudaMemsetAsync(E->d_dp, 0, sizeof(float) * S * 3 * NP, st));
        CK(cudaMemsetAsync(E->d_du, 0, sizeof(float) * S * 3 * NP, st));
    }
    return 0;
}

// A chunk's FP32 records to the caller's FP64 arrays; with host destinations they go down
// on the copy stream while the adjoint (or the next chunk) runs.
int chunk_records(SeisEngine* E, int first, int active, bool tan, double* result, double* result_diff,
                  cudaStream_t st)
{
    const long long per_shot = (long long)E->nt * E->nrec;
    store_records_kernel<<<grid_blocks(active * per_shot, 256), 256, 0, st>>>(first, active, per_shot, E->d_rec,
                                                                              result);
    E->launches++;
    if (tan) {
        store_records_kernel<<<grid_blocks(active * per_shot, 256), 256, 0, st>>>(first, active, per_shot,
                                                                                  E->d_drec, result_diff);
        E->launches++;
    }
    if (E->io.res || E->io.rd) {
        // host destinations: this chunk's records go down on the copy stream while
        // the adjoint (or the next chunk) runs
        const size_t off = (size_t)first * per_shot, n = sizeof(double) * (size_t)active * per_shot;
        CK(cudaEventRecord(E->io_ev, st));
        CK(cudaStreamWaitEvent(E->io_stream, E->io_ev, 0));
        if (E->io.res) CK(cudaMemcpyAsync(E->io.res + off, result + off, n, cudaMemcpyDeviceToHost, E->io_stream));
        if (E->io.rd && tan)
            CK(cudaMemcpyAsync(E->io.rd + off, result_diff + off, n, cudaMemcpyDeviceToHost, E->io_stream));
    }
    return 0;
}

// Seeds of a chunk's adjoint: the residual or the weights against its records, or (a
// Gauss-Newton matvec) its tangent records; zero adjoint fields for the tiled sweeps.
int chunk_seeds(SeisEngine* E, int first, int active, bool gn, int on_residual, const double* result,
                const double* vec_adjoint, bool zero_fields, cudaStream_t st)
{
    const long long NP = E->g.NP;
    const size_t S = (size_t)E->slots;
    const long long per_shot = (long long)E->nt * E->nrec;
    if (gn) {
        // seeds = the tangent records J v of these slots (FP32, as the records of a second call would be)
        CK(cudaMemcpyAsync(E->d_seed, E->d_drec, sizeof(float) * active * per_shot, cudaMemcpyDeviceToDevice,
                           st));
    } else {
        if (E->io.wait_va) {
            CK(cudaStreamWaitEvent(st, E->io_in_ev, 0));   // vec_adjoint's upload
            E->io.wait_va = false;
        }
        seeds_kernel<<<grid_blocks(active * per_shot, 256), 256, 0, st>>>(first, active, per_shot, on_residual,
                                                                          result, vec_adjoint, E->d_seed);
        E->launches++;
    }
    if (zero_fields) {
        CK(cudaMemsetAsync(E->d_lam, 0, sizeof(float) * S * 3 * NP, st));
        CK(cudaMemsetAsync(E->d_mu, 0, sizeof(float) * S * 3 * NP, st));
        CK(cudaMemsetAsync(E->d_gv, 0, sizeof(float) * S * NP, st));
        CK(cudaMemsetAsync(E->d_gk, 0, sizeof(float) * S * NP, st));
    }
    return 0;
}

// After the last chunk: the gradient folded back to the model grid with its min_vel
// entry, the misfit, and the error word's host mirror (in stream order after the sweeps).
int call_finish(SeisEngine* E, int nmodels, bool adj, const double* vec, const double* result,
                const double* vec_adjoint, double* result_adjoint, double* misfit, cudaStream_t st)
{
    const long long per_shot = (long long)E->nt * E->nrec;
    if (adj) {
        minvel_grad_kernel<<<nmodels, 1024, 0, st>>>(E->g, E->mg, E->d_dampx64, E->d_dampz64, E->d_acc_k,
                                                     result_adjoint);
        // the fold's row sums reuse acc_k (read above; NZ * nx <= NP per model)
        fold_rows_kernel<<<grid_blocks((long long)nmodels * E->g.NZ * E->nx, 256), 256, 0, st>>>(
            E->g, E->mg, nmodels, E->d_acc_v, E->d_acc_k);
        fold_cols_kernel<<<grid_blocks((long long)nmodels * E->nz * E->nx, 256), 256, 0, st>>>(
            E->g, E->mg, nmodels, vec, E->d_acc_k, result_adjoint);
        E->launches += 3;
        if (misfit) {
            // the partial sums reuse acc_v (read by the fold above; sized for kMisfitParts per model)
            misfit_partial_kernel<<<dim3(kMisfitParts / 128, nmodels), 128, 0, st>>>(E->nshots * per_shot, result,
                                                                                    vec_adjoint, E->d_acc_v);
            misfit_kernel<<<nmodels, kMisfitParts, 0, st>>>(E->d_acc_v, misfit);
            E->launches += 2;
        }
    }
    CK(cudaMemcpyAsync(E->h_err, E->d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaGetLastError());
    return 0;
}

}  // namespace

static int vel_to_seis_call(SeisEngine* E, int32_t nmodels, const double* vec, const double* vec_diff,
                            const double* vec_adjoint, int32_t on_residual, double* result, double* result_diff,
                            double* result_adjoint, double* misfit, void* stream, bool gn)
{
    E->err.clear();
    if (nmodels < 1 || nmodels > E->max_models)
        return E->fail(SEIS_E_INVALID, "nmodels=%d outside [1, %d]", nmodels, E->max_models);
    if (!vec || !result) return E->fail(SEIS_E_INVALID, "vec and result must be non-null");
    if ((vec_diff == nullptr) != (result_diff == nullptr))
        return E->fail(SEIS_E_INVALID, "result_diff must be given exactly when vec_diff is");
    if (!gn && (vec_adjoint == nullptr) != (result_adjoint == nullptr))
        return E->fail(SEIS_E_INVALID, "result_adjoint must be given exactly when vec_adjoint is");
    if (gn && (!vec_diff || !result_adjoint)) return E->fail(SEIS_E_INVALID, "a matvec needs vec_diff and result_adjoint");
    if (misfit && (!vec_adjoint || gn)) return E->fail(SEIS_E_INVALID, "misfit needs vec_adjoint");
    cudaStream_t st = (cudaStream_t)stream;
    const bool tan = vec_diff != nullptr, adj = vec_adjoint != nullptr || gn;
    const long long NP = E->g.NP;
    const size_t S = (size_t)E->slots;

    const bool ckmode = adj && E->ck > 0;
    {
        int rc = call_workspace(E, tan, adj, ckmode);
        if (rc) return rc;
    }

    int nev = 0;
    E->fwd_ev.clear();
    E->adj_ev.clear();
    E->adj_cl_ev.clear();
    auto rec_event = [&](int* idx, cudaStream_t on = nullptr) -> int {
        int r = next_event(E, idx);
        if (r) return r;
        CK(cudaEventRecord(E->ev_pool[*idx], on ? on : st));
        return 0;
    };

    E->last_stream = st;
    const bool wave = E->path == 3;     // persistent wavefront sweeps of the tiled kernels
    const SeisEngine::ClusterPlan* fplan = active_plan(E, false, tan);
    const bool cl_fwd = fplan && E->path != 1 && !wave && !ckmode;
    const SeisEngine::ClusterPlan* aplan = active_plan(E, true);
    const bool cl_adj = adj && aplan && E->path != 1 && !wave && !ckmode;
    E->last_fwd_launches = E->last_adj_launches = 0;
    E->last_adj_side = 0;
    E->last_fwd_side = 0;
    E->last_fwd_path = cl_fwd ? 2 : (wave ? 3 : 1);
    E->last_adj_path = adj ? (cl_adj ? 2 : (wave ? 3 : 1)) : 0;

    prep_models_kernel<<<grid_blocks((long long)nmodels * NP, 256), 256, 0, st>>>(
        E->g, E->mg, nmodels, vec, vec_diff, E->d_alpha, E->d_kfac, E->d_alpha_d, E->d_kdfac);
    E->launches++;
    if (adj) {
        CK(cudaMemsetAsync(E->d_acc_v, 0, sizeof(double) * nmodels * NP, st));
        CK(cudaMemsetAsync(E->d_acc_k, 0, sizeof(double) * nmodels * NP, st));
    }

    // sweeps are captured once per mode on the engine's private stream (the
    // caller's stream may be the legacy default stream, which cannot capture)
    if (ckmode && E->ck_graph_k != E->ck) {
        for (auto& gexec : E->ck_fwd_graph)
            if (gexec) { cudaGraphExecDestroy(gexec); gexec = nullptr; }
        if (E->ck_adj_graph) { cudaGraphExecDestroy(E->ck_adj_graph); E->ck_adj_graph = nullptr; }
        E->ck_graph_k = E->ck;
    }
    cudaGraphExec_t& fg = ckmode ? E->ck_fwd_graph[tan] : E->fwd_graph[tan][adj];
    if (!cl_fwd && !wave && !fg) {
        int r = ckmode ? capture_ck_fwd(E, tan, E->cap_stream, &fg) : capture_fwd(E, tan, adj, E->cap_stream, &fg);
        if (r) return r;
    }
    cudaGraphExec_t& ag = ckmode ? E->ck_adj_graph : E->adj_graph;
    if (adj && !cl_adj && !wave && !ag) {
        int r = ckmode ? capture_ck_adj(E, E->cap_stream, &ag) : capture_adj(E, E->cap_stream, &ag);
        if (r) return r;
    }
    // side adjoint: the last side_ns slots of a chunk run the tiled adjoint on the SMs
    // the adjoint clusters leave free; the clusters take the rest in whole rounds
    int side_s0 = (int)S, side_ns = 0;
    if (cl_adj)
        side_split(E, *aplan, (int)S, E->adj_side, aplan->shape->tmem ? kAdjTmClusterOverTiled : kAdjClusterOverTiled,
                   &side_s0, &side_ns);
    int fside_s0 = (int)S, fside_ns = 0;
    const bool fside_clusters = cl_fwd && side_cluster_plan(E, tan);   // split per chunk below (no graph)
    if (fside_clusters)
        side_split_clusters(*fplan, (int)S, E->fwd_side, E->fwd_side_clusters, kFwdSide8OverTm, &fside_s0, &fside_ns);
    else if (cl_fwd)
        side_split(E, *fplan, (int)S, E->fwd_side, tan ? kTanClusterOverTiled : kFwdClusterOverTiled, &fside_s0,
                   &fside_ns);
    // the tiled side sweeps' graphs of a split, captured on first use and kept
    auto side_graph = [&](bool fwd, int s0, int ns, cudaGraphExec_t* out) -> int {
        std::vector<SeisEngine::SideGraph>& cache = fwd ? E->fwd_side_graphs[tan][adj] : E->adj_side_graphs;
        for (const auto& e : cache)
            if (e.s0 == s0 && e.ns == ns) {
                *out = e.g;
                return 0;
            }
        if (cache.size() >= kMaxSideGraphs) {
            cudaGraphExecDestroy(cache.front().g);
            cache.erase(cache.begin());
        }
        int r = fwd ? capture_fwd_side(E, tan, adj, s0, ns, E->cap_stream, out)
                    : capture_adj_side(E, s0, ns, E->cap_stream, out);
        if (r) return r;
        cache.push_back({s0, ns, *out});
        return 0;
    };
    const int ncp = ckmode ? (E->nt + E->ck - 1) / E->ck : 0;

    const int total_shots = nmodels * E->nshots;
    // u buffer the forward graph was captured with
    float* ubuf = ckmode ? E->d_ring : (adj ? E->d_uhist : E->d_uring);
    const size_t ulevels = ckmode ? (size_t)E->ck + 1 : (adj ? (size_t)E->nt + 1 : 3);
    for (int first = 0; first < total_shots; first += (int)S) {
        const int active = std::min<int>((int)S, total_shots - first);
        {
            int r = chunk_begin(E, first, total_shots, active, vec, vec_diff, tan, ubuf, ulevels, st);
            if (r) return r;
        }
        int e0 = nev++;
        { int r = rec_event(&e0); if (r) return r; }
        if (cl_fwd && E->fwd_side < 0) {          // automatic: split this chunk's own shots
            if (fside_clusters)
                side_split_clusters(*fplan, active, -1, E->fwd_side_clusters, kFwdSide8OverTm, &fside_s0, &fside_ns);
            else
                side_split(E, *fplan, active, -1, tan ? kTanClusterOverTiled : kFwdClusterOverTiled, &fside_s0,
                           &fside_ns);
        }
        if (cl_adj && E->adj_side < 0)
            side_split(E, *aplan, active, -1, aplan->shape->tmem ? kAdjTmClusterOverTiled : kAdjClusterOverTiled,
                       &side_s0, &side_ns);
        if (cl_fwd && fside_ns && active > fside_s0) {
            // as the side adjoint: clusters on the high-priority stream over whole rounds,
            // the last slots' tiled forward on the low-priority one, joined back
            ClusterArgs ca = make_cluster_args(E, *fplan, adj);
            ca.slots = fside_s0;
            CK(cudaEventRecord(E->fork_ev, st));
            CK(cudaStreamWaitEvent(E->hi_stream, E->fork_ev, 0));
            CK(cudaStreamWaitEvent(E->side_stream, E->fork_ev, 0));
            int r = launch_cluster(E, fplan->shape->kernel, *fplan, fside_s0, ca, E->hi_stream);
            if (r) return r;
            const SeisEngine::ClusterPlan* sp = side_cluster_plan(E, tan);
            if (sp) {
                // the side slots on a few clusters of a smaller shape, beside the main ones
                ClusterArgs sa = make_cluster_args(E, *sp, adj);
                const long long per_shot_rec = (long long)E->nt * E->nrec;
                sa.shots += fside_s0;
                sa.smod += (long long)fside_s0 * E->nt;
                sa.rec += (long long)fside_s0 * per_shot_rec;
                if (sa.uhist) sa.uhist += (long long)fside_s0 * sa.u_slot_stride;
                sa.slots = active - fside_s0;
                SeisEngine::ClusterPlan few = *sp;
                few.nclusters = std::max(1, std::min(E->fwd_side_clusters, sp->nclusters));
                r = launch_cluster(E, sp->shape->kernel, few, sa.slots, sa, E->side_stream);
                if (r) return r;
            } else {
                cudaGraphExec_t sg = nullptr;
                r = side_graph(true, fside_s0, fside_ns, &sg);
                if (r) return r;
                CK(cudaGraphLaunch(sg, E->side_stream));
            }
            CK(cudaEventRecord(E->join_hi_ev, E->hi_stream));
            CK(cudaEventRecord(E->join_side_ev, E->side_stream));
            CK(cudaStreamWaitEvent(st, E->join_hi_ev, 0));
            CK(cudaStreamWaitEvent(st, E->join_side_ev, 0));
            const long long n = sp ? 1 : sweep_step_launches(E, true, false);
            E->launches += 1 + n;
            if (!sp) E->fwd_step_launches += n;
            E->last_fwd_launches += 1 + n;
            E->last_fwd_side += active - fside_s0;
        } else if (cl_fwd) {
            int r = launch_cluster(E, fplan->shape->kernel, *fplan, active, make_cluster_args(E, *fplan, adj), st);
            if (r) return r;
            E->launches += 1;
            E->last_fwd_launches += 1;
        } else if (wave) {
            int r = wave_sweep(E, tan ? 1 : 0, adj, ckmode, active, st);
            if (r) return r;
            E->last_fwd_launches += 1;
        } else {
            CK(cudaGraphLaunch(fg, st));
            const long long n = sweep_step_launches(E, true, ckmode);
            E->launches += n + 2 * ncp;
            E->fwd_step_launches += n;
            E->last_fwd_launches += n;
        }
        int e1 = nev++;
        { int r = rec_event(&e1); if (r) return r; }
        E->fwd_ev.push_back({e0, e1});
        {
            int r = chunk_records(E, first, active, tan, result, result_diff, st);
            if (r) return r;
        }
        if (adj) {
            {
                int r = chunk_seeds(E, first, active, gn, on_residual, result, vec_adjoint, !cl_adj, st);
                if (r) return r;
            }
            int a0 = nev++;
            { int r = rec_event(&a0); if (r) return r; }
            if (cl_adj && side_ns && active > side_s0) {
                // clusters on the high-priority stream (placed first), the side slots' tiled
                // adjoint on the low-priority one, both joined back before the gradient sums
                ClusterArgs ca = make_cluster_args(E, *aplan, true);
                ca.slots = side_s0;
                const long long off = (long long)side_s0 * NP;
                CK(cudaEventRecord(E->fork_ev, st));
                CK(cudaStreamWaitEvent(E->hi_stream, E->fork_ev, 0));
                CK(cudaStreamWaitEvent(E->side_stream, E->fork_ev, 0));
                int c0 = nev++, c1 = nev++;
                int r = rec_event(&c0, E->hi_stream);
                if (!r) r = launch_cluster(E, aplan->shape->kernel, *aplan, side_s0, ca, E->hi_stream);
                if (!r) r = rec_event(&c1, E->hi_stream);
                if (r) return r;
                E->adj_cl_ev.push_back({c0, c1});
                CK(cudaMemsetAsync(E->d_lam + 3 * off, 0, sizeof(float) * 3 * side_ns * NP, E->side_stream));
                CK(cudaMemsetAsync(E->d_mu + 3 * off, 0, sizeof(float) * 3 * side_ns * NP, E->side_stream));
                CK(cudaMemsetAsync(E->d_gv + off, 0, sizeof(float) * side_ns * NP, E->side_stream));
                CK(cudaMemsetAsync(E->d_gk + off, 0, sizeof(float) * side_ns * NP, E->side_stream));
                cudaGraphExec_t sg = nullptr;
                r = side_graph(false, side_s0, side_ns, &sg);
                if (r) return r;
                CK(cudaGraphLaunch(sg, E->side_stream));
                CK(cudaEventRecord(E->join_hi_ev, E->hi_stream));
                CK(cudaEventRecord(E->join_side_ev, E->side_stream));
                CK(cudaStreamWaitEvent(st, E->join_hi_ev, 0));
                CK(cudaStreamWaitEvent(st, E->join_side_ev, 0));
                const long long n = sweep_step_launches(E, false, false);
                E->launches += 1 + n;
                E->adj_step_launches += n;
                E->last_adj_launches += 1 + n;
                E->last_adj_side += active - side_s0;
            } else if (cl_adj) {
                int c0 = nev++, c1 = nev++;
                int r = rec_event(&c0);
                if (!r) r = launch_cluster(E, aplan->shape->kernel, *aplan, active, make_cluster_args(E, *aplan, true),
                                           st);
                if (!r) r = rec_event(&c1);
                if (r) return r;
                E->adj_cl_ev.push_back({c0, c1});
                E->launches += 1;
                E->last_adj_launches += 1;
            } else if (wave) {
                int r = wave_sweep(E, 2, true, ckmode, active, st);
                if (r) return r;
                E->last_adj_launches += 1;
            } else {
                CK(cudaGraphLaunch(ag, st));
                const long long n = sweep_step_launches(E, false, ckmode);
                E->launches += n + (ckmode ? 2 * ncp : 0);
                E->adj_step_launches += n;
                E->last_adj_launches += n;
            }
            int a1 = nev++;
            { int r = rec_event(&a1); if (r) return r; }
            E->adj_ev.push_back({a0, a1});
            accumulate_kernel<<<grid_blocks(NP, 256), 256, 0, st>>>(E->g, E->d_shots, (int)S, E->d_gv, E->d_gk,
                                                                    E->d_acc_v, E->d_acc_k);
            E->launches++;
        }
    }
    return call_finish(E, nmodels, adj, vec, result, vec_adjoint, result_adjoint, misfit, st);
}

// ---------------------------------------------------------------------------
// several engines' batches (models on different geometries) in one wavefront launch
// per sweep
// ---------------------------------------------------------------------------

extern "C" int seis_vel_to_seis_multi(int32_t n, SeisEngine* const* engines, const int32_t* nmodels,
                                      const double* const* vec, const double* const* vec_adjoint,
                                      int32_t on_residual, double* const* result, double* const* result_adjoint,
                                      double* const* misfit, void* stream)
{
    auto bad = [](const char* m) { set_thread_error(m); return SEIS_E_INVALID; };
    set_thread_error("");
    if (n < 1 || !engines || !nmodels || !vec || !result) return bad("seis_vel_to_seis_multi: empty or null arguments");
    if ((vec_adjoint == nullptr) != (result_adjoint == nullptr))
        return bad("seis_vel_to_seis_multi: result_adjoint must be given exactly when vec_adjoint is");
    if (misfit && !vec_adjoint) return bad("seis_vel_to_seis_multi: misfit needs vec_adjoint");
    std::vector<SeisEngine*> order(engines, engines + n);
    for (SeisEngine* E : order)
        if (!E) return bad("seis_vel_to_seis_multi: null engine");
    std::sort(order.begin(), order.end());
    if (std::adjacent_find(order.begin(), order.end()) != order.end())
        return bad("seis_vel_to_seis_multi: an engine appears twice (its workspace would be shared)");
    // every engine locked for the call, in address order
    std::vector<std::unique_lock<std::mutex>> locks;
    for (SeisEngine* E : order) locks.emplace_back(E->mu);
    const bool adj = vec_adjoint != nullptr;
    cudaStream_t st = (cudaStream_t)stream;
    SeisEngine* E0 = engines[0];
    auto fail = [&](int i, int rc) {
        set_thread_error(std::string("engine ") + std::to_string(i) + ": " + engines[i]->err);
        return rc;
    };
    int rounds = 0;
    for (int i = 0; i < n; ++i) {
        SeisEngine* E = engines[i];
        E->err.clear();
        if (nmodels[i] < 1 || nmodels[i] > E->max_models)
            return fail(i, E->fail(SEIS_E_INVALID, "nmodels=%d outside [1, %d]", nmodels[i], E->max_models));
        if (!vec[i] || !result[i] || (adj && (!vec_adjoint[i] || !result_adjoint[i])))
            return fail(i, E->fail(SEIS_E_INVALID, "null array"));
        for (const void* ptr : {(const void*)vec[i], (const void*)result[i],
                                adj ? (const void*)vec_adjoint[i] : nullptr, adj ? (const void*)result_adjoint[i] : nullptr,
                                misfit ? (const void*)misfit[i] : nullptr})
            if (host_ptr(ptr)) return fail(i, E->fail(SEIS_E_INVALID, "the multi-engine call takes device arrays only"));
        const bool ck = adj && E->ck > 0;
        int rc = call_workspace(E, false, adj, ck);
        if (rc) return fail(i, rc);
        E->io = SeisEngine::HostIO{};
        E->last_stream = st;
        E->fwd_ev.clear();
        E->adj_ev.clear();
        E->adj_cl_ev.clear();
        E->last_fwd_launches = E->last_adj_launches = 0;
        E->last_fwd_side = E->last_adj_side = 0;
        E->last_fwd_path = 3;
        E->last_adj_path = adj ? 3 : 0;
        const long long NP = E->g.NP;
        prep_models_kernel<<<grid_blocks((long long)nmodels[i] * NP, 256), 256, 0, st>>>(
            E->g, E->mg, nmodels[i], vec[i], nullptr, E->d_alpha, E->d_kfac, E->d_alpha_d, E->d_kdfac);
        E->launches++;
        if (adj) {
            if (cudaMemsetAsync(E->d_acc_v, 0, sizeof(double) * nmodels[i] * NP, st) != cudaSuccess ||
                cudaMemsetAsync(E->d_acc_k, 0, sizeof(double) * nmodels[i] * NP, st) != cudaSuccess)
                return fail(i, E->fail(SEIS_E_CUDA, "gradient accumulator reset failed"));
        }
        rounds = std::max(rounds, (nmodels[i] * E->nshots + E->slots - 1) / E->slots);
    }
    {
        int rc = wave_resident_mode(E0, 0);
        if (!rc && adj) rc = wave_resident_mode(E0, 2);
        if (rc) return fail(0, rc);
    }
    // round r sweeps chunk r of every engine that has one: one forward and one reverse launch
    for (int r = 0; r < rounds; ++r) {
        std::vector<int> part, first, active;
        for (int i = 0; i < n; ++i) {
            SeisEngine* E = engines[i];
            const int total = nmodels[i] * E->nshots, f = r * E->slots;
            if (f >= total) continue;
            part.push_back(i);
            first.push_back(f);
            active.push_back(std::min(E->slots, total - f));
        }
        for (size_t k = 0; k < part.size(); ++k) {
            SeisEngine* E = engines[part[k]];
            const bool ck = adj && E->ck > 0;
            float* ubuf = ck ? E->d_ring : (adj ? E->d_uhist : E->d_uring);
            const size_t ulevels = ck ? (size_t)E->ck + 1 : (adj ? (size_t)E->nt + 1 : 3);
            int rc = chunk_begin(E, first[k], nmodels[part[k]] * E->nshots, active[k], vec[part[k]], nullptr, false,
                                 ubuf, ulevels, st);
            if (rc) return fail(part[k], rc);
        }
        std::vector<WaveGroup> groups;
        std::vector<WaveArgs> args;
        for (size_t k = 0; k < part.size(); ++k) {
            SeisEngine* E = engines[part[k]];
            int rc = wave_groups(E, 0, adj, adj && E->ck > 0, active[k], wave_resident_of(E0, 0), groups, args, st);
            if (rc) return fail(part[k], rc);
            E->last_fwd_launches++;
        }
        {
            int rc = wave_launch(E0, 0, groups, args, st);
            if (rc) return fail(0, rc);
        }
        for (size_t k = 0; k < part.size(); ++k) {
            SeisEngine* E = engines[part[k]];
            int rc = chunk_records(E, first[k], active[k], false, result[part[k]], nullptr, st);
            if (!rc && adj)
                rc = chunk_seeds(E, first[k], active[k], false, on_residual, result[part[k]], vec_adjoint[part[k]],
                                 true, st);
            if (rc) return fail(part[k], rc);
        }
        if (!adj) continue;
        groups.clear();
        args.clear();
        for (size_t k = 0; k < part.size(); ++k) {
            SeisEngine* E = engines[part[k]];
            int rc = wave_groups(E, 2, true, E->ck > 0, active[k], wave_resident_of(E0, 2), groups, args, st);
            if (rc) return fail(part[k], rc);
            E->last_adj_launches++;
        }
        {
            int rc = wave_launch(E0, 2, groups, args, st);
            if (rc) return fail(0, rc);
        }
        for (size_t k = 0; k < part.size(); ++k) {
            SeisEngine* E = engines[part[k]];
            accumulate_kernel<<<grid_blocks(E->g.NP, 256), 256, 0, st>>>(E->g, E->d_shots, E->slots, E->d_gv, E->d_gk,
                                                                         E->d_acc_v, E->d_acc_k);
            E->launches++;
        }
    }
    for (int i = 0; i < n; ++i) {
        int rc = call_finish(engines[i], nmodels[i], adj, vec[i], result[i], adj ? vec_adjoint[i] : nullptr,
                             adj ? result_adjoint[i] : nullptr, misfit ? misfit[i] : nullptr, st);
        if (rc) return fail(i, rc);
    }
    return 0;
}
