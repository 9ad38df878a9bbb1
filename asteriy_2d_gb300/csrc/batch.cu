// batch.cu - many independent problems advanced together (the ast_batch_*
// entry points of include/asteriy_gb300.h).
//
// The problems are grouped into classes by (flux, recon), the two template
// parameters of the step code that differ between them; inside a class
// they are ordered by decreasing tile count.  A class owns one contiguous
// range of the device parameter arrays (one StepParams per problem, one
// array per ping-pong parity) and one tile prefix sum, and steps with one
// launch of batch_kernel over all of its problems' tiles.  Each problem has
// its own DevClock, so its dt reduction and funk_time shift stay its own
// (the last of its tiles to finish performs them; in the persistent batch
// kernel, the last CTA of the launch performs every problem's).
//
// Blocks of 16 steps are captured into one CUDA graph in which every class
// is an independent chain of launches: classes are forked from the caller's
// stream at the start of the block and joined at its end, so cheap (HLLC)
// and expensive (exact Godunov) classes overlap on the GPU.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <numeric>
#include <vector>

#include "../../include/asteriy_gb300.h"
#include "convert.cuh"
#include "launch.cuh"

using namespace ast;

namespace {

// Schedules of a class: 0..kNumShapes-1 one CTA per tile with tile shape
// kShapeTZ/kShapeTR[s]; kPersistent the persistent FP32 batch kernel (32x16
// tiles, the work list of shape 0); kPerProblem the single-problem
// persistent FP32 kernel once per problem, each problem its own stream
// (its own chain of launches in the step graph)
constexpr int kPersistent = kNumShapes, kPerProblem = kNumShapes + 1, kNumSchedules = kNumShapes + 2;
static_assert(kNumSchedules == AST_BATCH_SCHEDULES, "schedule count");

struct BatchClass {
    int flux, recon;
    int first, count;             // slots [first, first + count) of the parameter arrays
    int shape;                    // schedule in use
    int tiles[kNumSchedules];     // work-list length per schedule
    int ts_off[kNumSchedules];    // offset of its count+1 prefix sums in the tile_start array
    float ms[kNumSchedules];      // autotuner: ms per step per schedule (0: not timed)
    int grid;                     // persistent kernel: CTAs
    int work0;                    // persistent kernel: its first entry of the batch's work list
};

#define BATCH_CUDA(call)                                    \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
    } while (0)

int tiles_of(const ast_config& c, int shape)
{
    return ((c.N + kShapeTZ[shape] - 1) / kShapeTZ[shape]) * ((c.M + kShapeTR[shape] - 1) / kShapeTR[shape]);
}

}  // namespace

struct ast_batch {
    int nprob = 0;
    size_t elem = 8;
    std::vector<ast_config> cfg;        // user order
    std::vector<int> slot;              // user index -> parameter slot
    std::vector<long long> ld, plane;   // user order
    std::vector<size_t> off;            // user order: byte offset of time level 0 in the arena
    std::vector<size_t> level_bytes;    // user order: bytes of one time level
    std::vector<StepParams> hP;         // slot order, without state pointers
    std::vector<BatchClass> cls;
    void* arena = nullptr;
    DevClock* clocks = nullptr;         // user order
    StepParams* dP[2] = {nullptr, nullptr};
    int* tile_start = nullptr;
    double* stage_s = nullptr;
    double* stage_u = nullptr;
    float* mlp = nullptr;
    cudaStream_t stream = nullptr;
    std::vector<cudaStream_t> aux;      // one per class beyond the first
    std::vector<cudaEvent_t> ev;        // fork event + one join event per aux stream
    int cur = 0;
    cudaGraphExec_t graph = nullptr;
    int graph_steps = 0, graph_cur = -1;
    long long cells = 0;
    DevClock* clock_save = nullptr;     // autotuner: clocks saved around the trials
    int schedules = kNumShapes;         // schedules built for this precision
    CUtensorMap* maps = nullptr;        // FP32: per parity, load maps then store maps, slot order
    unsigned int* counters = nullptr;   // FP32: per class, then for the one-launch kernel, the persistent
                                        // kernel's two counters (claims, CTAs that left)
    BatchTile* work = nullptr;          // FP32: the persistent kernels' work list (every slot's 32x16 tiles,
                                        // slot order)
    int wait_polls = 0;                 // FP32: the shortest configured copy wait of the batch
    // FP32, per-problem schedule (slot order): host copies of the maps and
    // of each parity's parameters, CTAs, streams and join events
    std::vector<CUtensorMap> hmaps;
    std::vector<StepParams> hPp[2];
    std::vector<int> pgrid;
    std::vector<cudaStream_t> pstream;
    std::vector<cudaEvent_t> pev;
    cudaEvent_t pfork = nullptr;
    // FP32, one reconstruction: every problem in one launch of the mixed
    // kernel (32x16 tiles, slot order)
    bool mix_ok = false;
    int mixed = 0;                      // 1: steps are mixed launches, 2: persistent mixed launches
    int mix_grid = 0;                   // the persistent mixed kernel's CTAs
    int* mix_start = nullptr;           // prefix sums of the problems' tiles (nprob + 1), then
                                        // per slot the kernels' FLUX (nprob)
    int mix_tiles = 0, mix_recon = 0;
    float ms_mixed = 0.0f, ms_split = 0.0f;   // autotuner: ms per step, one launch (the faster mode) / per class
};

namespace {

void drop_graph(ast_batch* B)
{
    if (B->graph) {
        cudaGraphExecDestroy(B->graph);
        B->graph = nullptr;
    }
}

// parameter arrays of both parities (state pointers of each problem's two
// time levels) from the host copies
int upload_params(ast_batch* B)
{
    std::vector<StepParams> P(B->hP);
    for (int par = 0; par < 2; par++) {
        for (int i = 0; i < B->nprob; i++) {
            StepParams& p = P[B->slot[i]];
            char* base = (char*)B->arena + B->off[i];
            p.in = base + (par ? B->level_bytes[i] : 0);
            p.out = base + (par ? 0 : B->level_bytes[i]);
        }
        BATCH_CUDA(cudaMemcpy(B->dP[par], P.data(), sizeof(StepParams) * P.size(), cudaMemcpyHostToDevice));
        B->hPp[par] = P;
    }
    return AST_OK;
}

// one step of the problem in slot s with the single-problem persistent kernel
int launch_problem(ast_batch* B, const BatchClass& c, int s, cudaStream_t st)
{
    const size_t n = (size_t)B->nprob;
    return launch_step_tma(B->hPp[B->cur][s], B->hmaps[(2 * B->cur) * n + s], B->hmaps[(2 * B->cur + 1) * n + s],
                           c.flux, c.recon, B->pgrid[s], st, true, nullptr);
}

int launch_class(ast_batch* B, BatchClass& c, int shape, cudaStream_t st, bool launch)
{
    const StepParams* Ps = B->dP[B->cur] + c.first;
    const int* ts = B->tile_start + c.ts_off[shape];
    if (shape == kPerProblem) {
        if (!launch) {
            // the kernel's shared-memory limit, and each problem's CTAs
            int per_sm = 0, dev = 0, sms = 0;
            const size_t n = (size_t)B->nprob;
            int rc = launch_step_tma(B->hPp[0][c.first], B->hmaps[c.first], B->hmaps[n + c.first], c.flux, c.recon, 0,
                                     st, false, &per_sm);
            if (rc != AST_OK) return rc;
            BATCH_CUDA(cudaGetDevice(&dev));
            BATCH_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
            for (int s = c.first; s < c.first + c.count; s++) {
                const StepParams& P = B->hPp[0][s];
                const int tiles = ((P.N + kTmaTZ - 1) / kTmaTZ) * ((P.M + kTmaTR - 1) / kTmaTR);
                B->pgrid[s] = std::min(tiles, std::max(per_sm, 1) * sms);
            }
            return AST_OK;
        }
        // one step of every problem of the class, each on its stream
        BATCH_CUDA(cudaEventRecord(B->pfork, st));
        for (int s = c.first; s < c.first + c.count; s++) {
            BATCH_CUDA(cudaStreamWaitEvent(B->pstream[s], B->pfork, 0));
            const int rc = launch_problem(B, c, s, B->pstream[s]);
            if (rc != AST_OK) return rc;
            BATCH_CUDA(cudaEventRecord(B->pev[s], B->pstream[s]));
            BATCH_CUDA(cudaStreamWaitEvent(st, B->pev[s], 0));
        }
        return AST_OK;
    }
    if (shape == kPersistent) {
        // the class's run of the batch's work list; parameters and maps
        // indexed by slot
        const int ci = (int)(&c - B->cls.data());
        const CUtensorMap* tin = B->maps + (size_t)(2 * B->cur) * B->nprob;
        const CUtensorMap* tout = B->maps + (size_t)(2 * B->cur + 1) * B->nprob;
        if (!launch) {
            int per_sm = 0, dev = 0, sms = 0;
            int rc = launch_batch_tma(nullptr, nullptr, nullptr, nullptr, 0, 0, 0, nullptr, 0, c.flux, c.recon, 0,
                                      st, false, &per_sm);
            if (rc != AST_OK) return rc;
            BATCH_CUDA(cudaGetDevice(&dev));
            BATCH_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
            c.grid = std::min(c.tiles[shape], std::max(per_sm, 1) * sms);
            return AST_OK;
        }
        return launch_batch_tma(B->dP[B->cur], tin, tout, B->work + c.work0, c.tiles[shape], c.first, c.count,
                                B->counters + 2 * ci, B->wait_polls, c.flux, c.recon, c.grid, st, true, nullptr);
    }
    return launch_batch(B->elem, shape, Ps, ts, c.count, c.tiles[shape], c.flux, c.recon, st, launch);
}

// `count` steps of every class; classes beyond the first run on their own
// streams, forked from and joined back into `st`
int enqueue_steps(ast_batch* B, cudaStream_t st, int count)
{
    if (B->mixed == 2) {
        // the persistent one-launch kernel over every problem's tiles
        const size_t n = (size_t)B->nprob;
        unsigned int* counter = B->counters + 2 * B->cls.size();
        for (int i = 0; i < count; i++) {
            const int rc = launch_batch_tma_mixed(B->dP[B->cur], B->maps + (2 * B->cur) * n,
                                                  B->maps + (2 * B->cur + 1) * n, B->work, B->mix_tiles, B->nprob,
                                                  counter, B->wait_polls, B->mix_recon, B->mix_grid, st, true,
                                                  nullptr);
            if (rc != AST_OK) return rc;
            B->cur ^= 1;
        }
        return AST_OK;
    }
    if (B->mixed) {
        for (int i = 0; i < count; i++) {
            const int rc = launch_batch_mixed(B->dP[B->cur], B->mix_start, B->mix_start + B->nprob + 1, B->nprob,
                                              B->mix_tiles, B->mix_recon, st, true);
            if (rc != AST_OK) return rc;
            B->cur ^= 1;
        }
        return AST_OK;
    }
    const int nc = (int)B->cls.size();
    BATCH_CUDA(cudaEventRecord(B->ev[0], st));   // the fork point
    const int cur0 = B->cur;
    for (int c = 0; c < nc; c++) {
        BatchClass& k = B->cls[c];
        if (k.shape == kPerProblem) {
            // every problem of the class its own chain of `count` launches
            for (int s = k.first; s < k.first + k.count; s++) {
                cudaStream_t ps = B->pstream[s];
                BATCH_CUDA(cudaStreamWaitEvent(ps, B->ev[0], 0));
                B->cur = cur0;
                for (int i = 0; i < count; i++) {
                    const int rc = launch_problem(B, k, s, ps);
                    if (rc != AST_OK) {
                        B->cur = cur0;
                        return rc;
                    }
                    B->cur ^= 1;
                }
                BATCH_CUDA(cudaEventRecord(B->pev[s], ps));
                BATCH_CUDA(cudaStreamWaitEvent(st, B->pev[s], 0));
            }
            continue;
        }
        cudaStream_t sc = (c == 0) ? st : B->aux[c - 1];
        if (c > 0) BATCH_CUDA(cudaStreamWaitEvent(sc, B->ev[0], 0));
        B->cur = cur0;
        for (int i = 0; i < count; i++) {
            int rc = launch_class(B, k, k.shape, sc, true);
            if (rc != AST_OK) {
                B->cur = cur0;
                return rc;
            }
            B->cur ^= 1;
        }
        if (c > 0) {
            BATCH_CUDA(cudaEventRecord(B->ev[c], sc));
            BATCH_CUDA(cudaStreamWaitEvent(st, B->ev[c], 0));
        }
    }
    B->cur = cur0 ^ (count & 1);
    return AST_OK;
}

int capture_block(ast_batch* B, int count)
{
    drop_graph(B);
    cudaStream_t cs;
    BATCH_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    const int cur0 = B->cur;
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    int rc = AST_OK;
    if (e == cudaSuccess) {
        rc = enqueue_steps(B, cs, count);
        e = cudaStreamEndCapture(cs, &graph);
    }
    B->cur = cur0;
    cudaStreamDestroy(cs);
    if (e != cudaSuccess) return cuda_fail(e, "batch graph capture");
    if (rc != AST_OK) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    e = cudaGraphInstantiate(&B->graph, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
    B->graph_steps = count;
    B->graph_cur = cur0;
    return AST_OK;
}

bool bad_prob(const ast_batch* B, int prob) { return !B || prob < 0 || prob >= B->nprob; }

}  // namespace

extern "C" {

int ast_batch_create(const ast_config* cfgs, int nprob, ast_batch** out)
{
    if (!cfgs || !out || nprob < 1 || nprob > AST_BATCH_MAX) return set_error(AST_ERR_INVALID, "bad argument");
    *out = nullptr;
    for (int i = 0; i < nprob; i++) {
        const int rc = ast_config_check(&cfgs[i]);
        if (rc != AST_OK) return set_error(rc, "invalid problem configuration");
        if (cfgs[i].precision != cfgs[0].precision)
            return set_error(AST_ERR_INVALID, "all problems of a batch share one precision");
        if (cfgs[i].inflow_p > 0.0)
            return set_error(AST_ERR_UNSUPPORTED, "the characteristic inflow is a single-problem option");
        if (cfgs[i].flux == AST_FLUX_HLLCQ)
            return set_error(AST_ERR_UNSUPPORTED, "the HLLCQ flux is a single-problem option");
    }
    ast_batch* B = new (std::nothrow) ast_batch();
    if (!B) return set_error(AST_ERR_NOMEM, "host allocation");
    B->nprob = nprob;
    B->elem = (cfgs[0].precision == AST_PREC_FP32) ? 4 : 8;
    B->cfg.assign(cfgs, cfgs + nprob);
    B->ld.resize(nprob);
    B->plane.resize(nprob);
    B->off.resize(nprob);
    B->level_bytes.resize(nprob);
    B->slot.resize(nprob);

    // arena layout: per problem two time levels of four planes, each level
    // 256-byte aligned, rows padded to 128 bytes
    size_t total = 0, maxK = 0;
    const long long align = 128 / (long long)B->elem;
    for (int i = 0; i < nprob; i++) {
        const ast_config& c = B->cfg[i];
        B->ld[i] = ((long long)c.N + align - 1) / align * align;
        B->plane[i] = B->ld[i] * c.M;
        B->level_bytes[i] = ((size_t)B->plane[i] * 4 * B->elem + 255) / 256 * 256;
        B->off[i] = total;
        total += 2 * B->level_bytes[i];
        maxK = std::max(maxK, (size_t)c.N * c.M);
        B->cells += (long long)c.N * c.M;
    }

    // classes by (flux, recon); inside a class, larger problems first
    std::vector<int> order(nprob);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        const ast_config &x = B->cfg[a], &y = B->cfg[b];
        if (x.flux != y.flux) return x.flux > y.flux;   // exact Godunov first
        if (x.recon != y.recon) return x.recon > y.recon;
        return (long long)x.N * x.M > (long long)y.N * y.M;
    });
    for (int s = 0; s < nprob; s++) {
        const ast_config& c = B->cfg[order[s]];
        if (B->cls.empty() || B->cls.back().flux != c.flux || B->cls.back().recon != c.recon) {
            BatchClass k;
            std::memset(&k, 0, sizeof k);
            k.flux = c.flux;
            k.recon = c.recon;
            k.first = s;
            B->cls.push_back(k);
        }
        B->cls.back().count++;
        B->slot[order[s]] = s;
    }
    // work lists: per class and tile shape, the prefix sums of its problems'
    // tile counts (count + 1 entries); the persistent kernel uses shape 0's
    std::vector<int> ts_host;
    for (BatchClass& k : B->cls) {
        for (int sh = 0; sh < kNumShapes; sh++) {
            k.ts_off[sh] = (int)ts_host.size();
            ts_host.push_back(0);
            for (int s = k.first; s < k.first + k.count; s++) {
                k.tiles[sh] += tiles_of(B->cfg[order[s]], sh);
                ts_host.push_back(k.tiles[sh]);
            }
        }
        k.ts_off[kPersistent] = k.ts_off[kPerProblem] = k.ts_off[0];
        k.tiles[kPersistent] = k.tiles[kPerProblem] = k.tiles[0];
    }
    if (B->elem == 4) B->schedules = kNumSchedules;

    cudaError_t e;
    const size_t nts = ts_host.size();
    if ((e = cudaMalloc(&B->arena, total)) != cudaSuccess ||
        (e = cudaMalloc(&B->clocks, sizeof(DevClock) * nprob)) != cudaSuccess ||
        (e = cudaMalloc(&B->clock_save, sizeof(DevClock) * nprob)) != cudaSuccess ||
        (e = cudaMalloc(&B->dP[0], sizeof(StepParams) * nprob)) != cudaSuccess ||
        (e = cudaMalloc(&B->dP[1], sizeof(StepParams) * nprob)) != cudaSuccess ||
        (e = cudaMalloc(&B->tile_start, sizeof(int) * nts)) != cudaSuccess ||
        (e = cudaMalloc(&B->stage_s, maxK * 2 * sizeof(double))) != cudaSuccess ||
        (e = cudaMalloc(&B->stage_u, maxK * 2 * sizeof(double))) != cudaSuccess) {
        ast_batch_destroy(B);
        set_error(AST_ERR_NOMEM, "batch device allocation");
        return AST_ERR_NOMEM;
    }
    int rc = AST_OK;
    if ((e = cudaMemset(B->arena, 0, total)) != cudaSuccess ||
        (e = cudaMemcpy(B->tile_start, ts_host.data(), sizeof(int) * nts, cudaMemcpyHostToDevice)) != cudaSuccess)
        rc = cuda_fail(e, "batch initialisation");
    std::vector<DevClock> clk(nprob);
    B->hP.resize(nprob);
    for (int i = 0; i < nprob && rc == AST_OK; i++) {
        std::memset(&clk[i], 0, sizeof(DevClock));
        clk[i].T_do = B->cfg[i].dt_first;
        StepParams& p = B->hP[B->slot[i]];
        fill_step_params(p, B->cfg[i]);
        p.ld = B->ld[i];
        p.plane = B->plane[i];
        p.clock = B->clocks + i;
    }
    if (rc == AST_OK &&
        (e = cudaMemcpy(B->clocks, clk.data(), sizeof(DevClock) * nprob, cudaMemcpyHostToDevice)) != cudaSuccess)
        rc = cuda_fail(e, "batch clocks");
    if (rc == AST_OK) rc = upload_params(B);
    if (rc == AST_OK && B->schedules > kNumShapes) {
        // FP32: tensor maps of every problem's two time levels (tile-box
        // loads with halo, tile stores), slot order, and the tile counters
        std::vector<CUtensorMap> maps((size_t)4 * nprob);
        for (int i = 0; i < nprob && rc == AST_OK; i++) {
            const int sl = B->slot[i];
            for (int par = 0; par < 2 && rc == AST_OK; par++) {
                char* base = (char*)B->arena + B->off[i];
                void* lin = base + (par ? B->level_bytes[i] : 0);
                void* lout = base + (par ? 0 : B->level_bytes[i]);
                rc = encode_planes(&maps[(size_t)(2 * par) * nprob + sl], lin, B->cfg[i], B->ld[i], B->plane[i],
                                   kTmaTZ + 8, kTmaTR + 4);
                if (rc == AST_OK)
                    rc = encode_planes(&maps[(size_t)(2 * par + 1) * nprob + sl], lout, B->cfg[i], B->ld[i],
                                       B->plane[i], kTmaTZ, kTmaTR);
            }
        }
        B->hmaps = maps;
        // the persistent kernels' work list: every slot's 32x16 tiles in
        // slot order (each class a contiguous run of it)
        std::vector<BatchTile> work;
        for (BatchClass& k : B->cls) {
            k.work0 = (int)work.size();
            for (int s = k.first; s < k.first + k.count; s++) {
                const ast_config& c = B->cfg[order[s]];
                const int fk = (c.flux == AST_FLUX_HLL) ? 0 : (c.flux == AST_FLUX_HLLC) ? 1
                                                          : (c.flux == AST_FLUX_HLLC_A) ? 3 : 2;
                const int tz = (c.N + kTmaTZ - 1) / kTmaTZ;
                const int nt = tz * ((c.M + kTmaTR - 1) / kTmaTR);
                for (int t = 0; t < nt; t++) {
                    BatchTile e;
                    std::memset(&e, 0, sizeof e);
                    e.sf = s | (fk << 24);
                    e.n0 = (t % tz) * kTmaTZ;
                    e.m0 = (t / tz) * kTmaTR;
                    e.clock = B->clocks + order[s];
                    work.push_back(e);
                }
            }
        }
        B->wait_polls = tma::kWaitLimit;
        for (int i = 0; i < nprob; i++)
            if (B->cfg[i].copy_wait_polls > 0) B->wait_polls = std::min(B->wait_polls, B->cfg[i].copy_wait_polls);
        B->pgrid.assign(nprob, 0);
        for (int s = 0; s < nprob && rc == AST_OK; s++) {
            cudaStream_t ps;
            cudaEvent_t pe;
            if ((e = cudaStreamCreateWithFlags(&ps, cudaStreamNonBlocking)) != cudaSuccess) {
                rc = cuda_fail(e, "batch problem stream");
                break;
            }
            B->pstream.push_back(ps);
            if ((e = cudaEventCreateWithFlags(&pe, cudaEventDisableTiming)) != cudaSuccess) {
                rc = cuda_fail(e, "batch problem event");
                break;
            }
            B->pev.push_back(pe);
        }
        if (rc == AST_OK && (e = cudaEventCreateWithFlags(&B->pfork, cudaEventDisableTiming)) != cudaSuccess)
            rc = cuda_fail(e, "batch fork event");
        const size_t ncnt = 2 * (B->cls.size() + 1);
        if (rc == AST_OK && ((e = cudaMalloc(&B->maps, sizeof(CUtensorMap) * maps.size())) != cudaSuccess ||
                             (e = cudaMalloc(&B->counters, sizeof(unsigned int) * ncnt)) != cudaSuccess ||
                             (e = cudaMalloc(&B->work, sizeof(BatchTile) * work.size())) != cudaSuccess ||
                             (e = cudaMemcpy(B->maps, maps.data(), sizeof(CUtensorMap) * maps.size(),
                                             cudaMemcpyHostToDevice)) != cudaSuccess ||
                             (e = cudaMemcpy(B->work, work.data(), sizeof(BatchTile) * work.size(),
                                             cudaMemcpyHostToDevice)) != cudaSuccess ||
                             (e = cudaMemset(B->counters, 0, sizeof(unsigned int) * ncnt)) != cudaSuccess))
            rc = cuda_fail(e, "batch tensor maps");
        // the persistent kernel is the FP32 default
        for (BatchClass& k : B->cls) k.shape = kPersistent;
    }
    for (size_t c = 0; c < B->cls.size() && rc == AST_OK; c++)
        for (int sh = 0; sh < B->schedules && rc == AST_OK; sh++) rc = launch_class(B, B->cls[c], sh, nullptr, false);
    // the one-launch work list (FP32, when every problem has the same
    // reconstruction): every slot's 32x16 tiles
    B->mix_ok = B->elem == 4;
    for (int i = 1; i < nprob; i++)
        if (cfgs[i].recon != cfgs[0].recon) B->mix_ok = false;
    if (rc == AST_OK && B->mix_ok) {
        std::vector<int> ms(2 * nprob + 1, 0);
        for (int s = 0; s < nprob; s++) {
            const ast_config& c = B->cfg[order[s]];
            ms[s + 1] = ms[s] + tiles_of(c, 0);
            ms[nprob + 1 + s] =
                (c.flux == AST_FLUX_HLL) ? 0 : (c.flux == AST_FLUX_HLLC) ? 1 : (c.flux == AST_FLUX_HLLC_A) ? 3 : 2;
        }
        B->mix_tiles = ms[nprob];
        B->mix_recon = cfgs[0].recon;
        if ((e = cudaMalloc(&B->mix_start, sizeof(int) * ms.size())) != cudaSuccess ||
            (e = cudaMemcpy(B->mix_start, ms.data(), sizeof(int) * ms.size(), cudaMemcpyHostToDevice)) != cudaSuccess)
            rc = cuda_fail(e, "batch work list");
        if (rc == AST_OK) rc = launch_batch_mixed(nullptr, nullptr, nullptr, 0, 0, B->mix_recon, nullptr, false);
        if (rc == AST_OK) {
            // the persistent one-launch kernel: as many CTAs as fit, at most
            // one per tile
            int per_sm = 0, dev = 0, sms = 0;
            rc = launch_batch_tma_mixed(nullptr, nullptr, nullptr, nullptr, 0, 0, nullptr, 0, B->mix_recon, 0,
                                        nullptr, false, &per_sm);
            if (rc == AST_OK && (e = cudaGetDevice(&dev)) != cudaSuccess) rc = cuda_fail(e, "cudaGetDevice");
            if (rc == AST_OK && (e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
                rc = cuda_fail(e, "cudaDeviceGetAttribute");
            if (rc == AST_OK) B->mix_grid = std::min(B->mix_tiles, std::max(per_sm, 1) * sms);
        }
    }
    for (size_t c = 1; c < B->cls.size() && rc == AST_OK; c++) {
        cudaStream_t s;
        if ((e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)) != cudaSuccess) {
            rc = cuda_fail(e, "batch stream");
            break;
        }
        B->aux.push_back(s);
    }
    for (size_t c = 0; c < B->cls.size() && rc == AST_OK; c++) {
        cudaEvent_t ev;
        if ((e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess) {
            rc = cuda_fail(e, "batch event");
            break;
        }
        B->ev.push_back(ev);
    }
    if (rc != AST_OK) {
        ast_batch_destroy(B);
        return rc;
    }
    *out = B;
    return AST_OK;
}

int ast_batch_destroy(ast_batch* B)
{
    if (!B) return AST_OK;
    drop_graph(B);
    for (cudaStream_t s : B->aux) cudaStreamDestroy(s);
    for (cudaStream_t s : B->pstream) cudaStreamDestroy(s);
    for (cudaEvent_t e : B->pev) cudaEventDestroy(e);
    if (B->pfork) cudaEventDestroy(B->pfork);
    for (cudaEvent_t e : B->ev) cudaEventDestroy(e);
    cudaFree(B->arena);
    cudaFree(B->clocks);
    cudaFree(B->clock_save);
    cudaFree(B->maps);
    cudaFree(B->counters);
    cudaFree(B->work);
    cudaFree(B->dP[0]);
    cudaFree(B->dP[1]);
    cudaFree(B->tile_start);
    cudaFree(B->mix_start);
    cudaFree(B->stage_s);
    cudaFree(B->stage_u);
    cudaFree(B->mlp);
    delete B;
    return AST_OK;
}

int ast_batch_set_stream(ast_batch* B, void* stream)
{
    if (!B) return set_error(AST_ERR_INVALID, "null batch");
    B->stream = (cudaStream_t)stream;
    drop_graph(B);
    return AST_OK;
}

int ast_batch_set_state(ast_batch* B, int prob, const double* s, const double* u, int on_device)
{
    if (bad_prob(B, prob) || !s || !u) return set_error(AST_ERR_INVALID, "bad argument");
    const ast_config& c = B->cfg[prob];
    const long long K = (long long)c.N * c.M;
    const size_t bytes = (size_t)K * 2 * sizeof(double);
    const double* ds = s;
    const double* du = u;
    if (!on_device) {
        BATCH_CUDA(cudaMemcpyAsync(B->stage_s, s, bytes, cudaMemcpyHostToDevice, B->stream));
        BATCH_CUDA(cudaMemcpyAsync(B->stage_u, u, bytes, cudaMemcpyHostToDevice, B->stream));
        ds = B->stage_s;
        du = B->stage_u;
    }
    void* dst = (char*)B->arena + B->off[prob] + (B->cur ? B->level_bytes[prob] : 0);
    const int nb = (int)((K + 255) / 256);
    if (B->elem == 8)
        aos_to_soa<double><<<nb, 256, 0, B->stream>>>((const double2*)ds, (const double2*)du, (double*)dst, c.N, c.M,
                                                      B->ld[prob], B->plane[prob]);
    else
        aos_to_soa<float><<<nb, 256, 0, B->stream>>>((const double2*)ds, (const double2*)du, (float*)dst, c.N, c.M,
                                                     B->ld[prob], B->plane[prob]);
    BATCH_CUDA(cudaGetLastError());
    if (!on_device) BATCH_CUDA(cudaStreamSynchronize(B->stream));
    return AST_OK;
}

int ast_batch_get_state(ast_batch* B, int prob, double* s, double* u, int on_device)
{
    if (bad_prob(B, prob) || !s || !u) return set_error(AST_ERR_INVALID, "bad argument");
    const ast_config& c = B->cfg[prob];
    const long long K = (long long)c.N * c.M;
    double* ds = on_device ? s : B->stage_s;
    double* du = on_device ? u : B->stage_u;
    const void* src = (const char*)B->arena + B->off[prob] + (B->cur ? B->level_bytes[prob] : 0);
    const int nb = (int)((K + 255) / 256);
    if (B->elem == 8)
        soa_to_aos<double><<<nb, 256, 0, B->stream>>>((const double*)src, (double2*)ds, (double2*)du, c.N, c.M,
                                                      B->ld[prob], B->plane[prob]);
    else
        soa_to_aos<float><<<nb, 256, 0, B->stream>>>((const float*)src, (double2*)ds, (double2*)du, c.N, c.M,
                                                     B->ld[prob], B->plane[prob]);
    BATCH_CUDA(cudaGetLastError());
    if (!on_device) {
        const size_t bytes = (size_t)K * 2 * sizeof(double);
        BATCH_CUDA(cudaMemcpyAsync(s, ds, bytes, cudaMemcpyDeviceToHost, B->stream));
        BATCH_CUDA(cudaMemcpyAsync(u, du, bytes, cudaMemcpyDeviceToHost, B->stream));
        BATCH_CUDA(cudaStreamSynchronize(B->stream));
    }
    return AST_OK;
}

int ast_batch_set_clock(ast_batch* B, int prob, double T_do, double TT, int64_t step)
{
    if (bad_prob(B, prob)) return set_error(AST_ERR_INVALID, "bad argument");
    DevClock c;
    BATCH_CUDA(cudaMemcpyAsync(&c, B->clocks + prob, sizeof c, cudaMemcpyDeviceToHost, B->stream));
    BATCH_CUDA(cudaStreamSynchronize(B->stream));
    c.T_do = T_do;
    c.TT = TT;
    c.step = step;
    c.smax_z = c.smax_r = 0;
    c.done = 0;
    BATCH_CUDA(cudaMemcpyAsync(B->clocks + prob, &c, sizeof c, cudaMemcpyHostToDevice, B->stream));
    BATCH_CUDA(cudaStreamSynchronize(B->stream));
    return AST_OK;
}

int ast_batch_get_clock(ast_batch* B, int prob, double* T_do, double* TT, int64_t* step)
{
    if (bad_prob(B, prob)) return set_error(AST_ERR_INVALID, "bad argument");
    DevClock c;
    BATCH_CUDA(cudaMemcpyAsync(&c, B->clocks + prob, sizeof c, cudaMemcpyDeviceToHost, B->stream));
    BATCH_CUDA(cudaStreamSynchronize(B->stream));
    if (T_do) *T_do = c.T_do;
    if (TT) *TT = c.TT;
    if (step) *step = c.step;
    return AST_OK;
}

int ast_batch_step(ast_batch* B, int nsteps)
{
    if (!B || nsteps < 0) return set_error(AST_ERR_INVALID, "bad argument");
    for (int i = 0; i < B->nprob; i++) {
        const ast_config& c = B->cfg[i];
        if (c.flux == AST_FLUX_GODUNOV && c.guess == AST_GUESS_MLP && B->hP[B->slot[i]].riemann_newton && !B->mlp)
            return set_error(AST_ERR_INVALID, "guess == MLP needs ast_batch_set_mlp first");
    }
    // a block of an even number of steps returns to the same buffers, so
    // one captured block is replayed back to back
    const int block = 16;
    while (nsteps >= block) {
        if (!B->graph || B->graph_steps != block || B->graph_cur != B->cur) {
            const int rc = capture_block(B, block);
            if (rc != AST_OK) return rc;
        }
        BATCH_CUDA(cudaGraphLaunch(B->graph, B->stream));
        nsteps -= block;
    }
    if (nsteps > 0) {
        const int cur0 = B->cur;
        const int rc = enqueue_steps(B, B->stream, nsteps);
        if (rc != AST_OK) return rc;
        B->cur = cur0 ^ (nsteps & 1);
    }
    return AST_OK;
}

int ast_batch_synchronize(ast_batch* B)
{
    if (!B) return set_error(AST_ERR_INVALID, "null batch");
    BATCH_CUDA(cudaStreamSynchronize(B->stream));
    std::vector<DevClock> c(B->nprob);
    BATCH_CUDA(cudaMemcpy(c.data(), B->clocks, sizeof(DevClock) * B->nprob, cudaMemcpyDeviceToHost));
    for (const DevClock& k : c)
        if (k.status & AST_ST_NONFINITE) return set_error(AST_ERR_NUMERIC, "non-finite wave speed");
    for (const DevClock& k : c) {
        if (k.status & AST_ST_TIMEOUT) return set_error(AST_ERR_CUDA, "a bulk tile copy did not arrive in time");
    }
    return AST_OK;
}

int ast_batch_get_stats(ast_batch* B, int prob, ast_stats* out, int reset)
{
    if (bad_prob(B, prob) || !out) return set_error(AST_ERR_INVALID, "bad argument");
    DevClock c;
    BATCH_CUDA(cudaMemcpyAsync(&c, B->clocks + prob, sizeof c, cudaMemcpyDeviceToHost, B->stream));
    BATCH_CUDA(cudaStreamSynchronize(B->stream));
    std::memset(out, 0, sizeof *out);
    out->status = c.status;
    out->rho_floor = c.cnt[0];
    out->p_floor = c.cnt[1];
    out->newton_calls = c.cnt[2];
    out->newton_iters = c.cnt[3];
    out->bisect_calls = c.cnt[4];
    out->bisect_iters = c.cnt[5];
    out->mlp_fallback = c.cnt[6];
    out->newton_max_iters = (uint32_t)c.cnt[7];
    out->strong_calls = c.cnt[8];
    out->strong_iters = c.cnt[9];
    if (reset) {
        c.status = 0;
        std::memset(c.cnt, 0, sizeof c.cnt);
        BATCH_CUDA(cudaMemcpyAsync(B->clocks + prob, &c, sizeof c, cudaMemcpyHostToDevice, B->stream));
        BATCH_CUDA(cudaStreamSynchronize(B->stream));
    }
    return AST_OK;
}

int ast_batch_set_mlp(ast_batch* B, const float* params)
{
    if (!B || !params) return set_error(AST_ERR_INVALID, "null argument");
    // the parameter arrays may be in use by queued steps
    BATCH_CUDA(cudaStreamSynchronize(B->stream));
    // the parameter block and, after it, its packed form for the step kernels
    if (!B->mlp) BATCH_CUDA(cudaMalloc(&B->mlp, sizeof(float) * kMlpDevFloats));
    BATCH_CUDA(cudaMemcpy(B->mlp, params, sizeof(float) * AST_MLP_NPARAM, cudaMemcpyHostToDevice));
    const int rc = launch_mlp_pack(B->mlp, B->stream);
    if (rc != AST_OK) return rc;
    BATCH_CUDA(cudaStreamSynchronize(B->stream));
    for (StepParams& p : B->hP) p.mlp = B->mlp;
    drop_graph(B);
    return upload_params(B);
}

int ast_batch_info(ast_batch* B, int64_t* cells, int64_t* tiles, int* launches_per_step)
{
    if (!B) return set_error(AST_ERR_INVALID, "null batch");
    if (cells) *cells = B->cells;
    if (tiles) {
        *tiles = 0;
        if (B->mixed) *tiles = B->mix_tiles;
        else
            for (const BatchClass& k : B->cls) *tiles += k.tiles[k.shape];
    }
    if (launches_per_step) *launches_per_step = B->mixed ? 1 : (int)B->cls.size();
    return AST_OK;
}

int ast_batch_num_classes(ast_batch* B)
{
    if (!B) return set_error(AST_ERR_INVALID, "null batch");
    return (int)B->cls.size();
}

int ast_batch_set_mixed(ast_batch* B, int on)
{
    if (!B || on < 0 || on > 2) return set_error(AST_ERR_INVALID, "bad argument");
    if (on && !B->mix_ok)
        return set_error(AST_ERR_UNSUPPORTED, "one launch needs FP32 problems with one reconstruction");
    B->mixed = on;
    drop_graph(B);
    return AST_OK;
}

int ast_batch_get_mixed(ast_batch* B, int* on, float* ms_mixed, float* ms_split)
{
    if (!B) return set_error(AST_ERR_INVALID, "null batch");
    if (on) *on = B->mixed;
    if (ms_mixed) *ms_mixed = B->ms_mixed;
    if (ms_split) *ms_split = B->ms_split;
    return AST_OK;
}

int ast_batch_class(ast_batch* B, int cls, int* flux, int* recon, int* nprob, int* schedule, int* tile_z,
                    int* tile_r, float* ms_per_schedule)
{
    if (!B || cls < 0 || cls >= (int)B->cls.size()) return set_error(AST_ERR_INVALID, "bad argument");
    const BatchClass& k = B->cls[cls];
    const int shape = (k.shape >= kNumShapes) ? 0 : k.shape;   // the persistent schedules tile 32x16
    if (flux) *flux = k.flux;
    if (recon) *recon = k.recon;
    if (nprob) *nprob = k.count;
    if (schedule) *schedule = k.shape;
    if (tile_z) *tile_z = kShapeTZ[shape];
    if (tile_r) *tile_r = kShapeTR[shape];
    if (ms_per_schedule)
        for (int sh = 0; sh < kNumSchedules; sh++) ms_per_schedule[sh] = (sh < B->schedules) ? k.ms[sh] : 0.0f;
    return AST_OK;
}

int ast_batch_set_schedule(ast_batch* B, int cls, int schedule)
{
    if (!B || cls < 0 || cls >= (int)B->cls.size() || schedule < 0 || schedule >= AST_BATCH_SCHEDULES)
        return set_error(AST_ERR_INVALID, "bad argument");
    if (schedule >= B->schedules) return set_error(AST_ERR_UNSUPPORTED, "schedule not built for this precision");
    B->cls[cls].shape = schedule;
    drop_graph(B);
    return AST_OK;
}

int ast_batch_set_tiles(ast_batch* B, int cls, int tile_z, int tile_r)
{
    if (!B || cls < 0 || cls >= (int)B->cls.size()) return set_error(AST_ERR_INVALID, "bad argument");
    for (int sh = 0; sh < kNumShapes; sh++)
        if (kShapeTZ[sh] == tile_z && kShapeTR[sh] == tile_r) return ast_batch_set_schedule(B, cls, sh);
    return set_error(AST_ERR_UNSUPPORTED, "tile shape not built");
}

int ast_batch_autotune(ast_batch* B, int trials)
{
    if (!B || trials < 1) return set_error(AST_ERR_INVALID, "bad argument");
    // every trial step reads the current time level and writes the other
    // one, so the state is left as it was; the clocks (dt, time, counters)
    // are saved first and put back afterwards
    cudaEvent_t e0, e1;
    BATCH_CUDA(cudaEventCreate(&e0));
    BATCH_CUDA(cudaEventCreate(&e1));
    int rc = AST_OK;
    cudaError_t e = cudaMemcpyAsync(B->clock_save, B->clocks, sizeof(DevClock) * B->nprob,
                                    cudaMemcpyDeviceToDevice, B->stream);
    if (e != cudaSuccess) rc = cuda_fail(e, "autotune clock save");
    for (BatchClass& k : B->cls) {
        float best = 0.0f;
        for (int sh = 0; sh < B->schedules && rc == AST_OK; sh++) {
            rc = launch_class(B, k, sh, B->stream, true);   // warm-up
            if (rc == AST_OK && (e = cudaEventRecord(e0, B->stream)) != cudaSuccess) rc = cuda_fail(e, "event");
            for (int t = 0; t < trials && rc == AST_OK; t++) rc = launch_class(B, k, sh, B->stream, true);
            if (rc == AST_OK && (e = cudaEventRecord(e1, B->stream)) != cudaSuccess) rc = cuda_fail(e, "event");
            if (rc == AST_OK && (e = cudaEventSynchronize(e1)) != cudaSuccess) rc = cuda_fail(e, "event");
            float ms = 0.0f;
            if (rc == AST_OK && (e = cudaEventElapsedTime(&ms, e0, e1)) != cudaSuccess) rc = cuda_fail(e, "event");
            if (rc != AST_OK) break;
            k.ms[sh] = ms / trials;
            if (sh == 0 || k.ms[sh] < best) {
                best = k.ms[sh];
                k.shape = sh;
            }
        }
    }
    // then the whole step: the classes' chosen schedules (one launch per
    // class, concurrent chains) against every problem in one launch
    if (rc == AST_OK && B->mix_ok) {
        const int cur0 = B->cur;
        float ms2[3] = {0.0f, 0.0f, 0.0f};
        for (int mode = 0; mode < 3 && rc == AST_OK; mode++) {
            B->mixed = mode;
            rc = enqueue_steps(B, B->stream, 1);   // warm-up
            B->cur = cur0;
            if (rc == AST_OK && (e = cudaEventRecord(e0, B->stream)) != cudaSuccess) rc = cuda_fail(e, "event");
            for (int t = 0; t < trials && rc == AST_OK; t++) {
                rc = enqueue_steps(B, B->stream, 1);
                B->cur = cur0;
            }
            if (rc == AST_OK && (e = cudaEventRecord(e1, B->stream)) != cudaSuccess) rc = cuda_fail(e, "event");
            if (rc == AST_OK && (e = cudaEventSynchronize(e1)) != cudaSuccess) rc = cuda_fail(e, "event");
            if (rc == AST_OK && (e = cudaEventElapsedTime(&ms2[mode], e0, e1)) != cudaSuccess) rc = cuda_fail(e, "event");
        }
        B->cur = cur0;
        B->ms_split = ms2[0] / trials;
        // the faster of the two one-launch modes against the classes' launches
        const int one = (ms2[2] < ms2[1]) ? 2 : 1;
        B->ms_mixed = ms2[one] / trials;
        B->mixed = (rc == AST_OK && B->ms_mixed < B->ms_split) ? one : 0;
    }
    e = cudaMemcpyAsync(B->clocks, B->clock_save, sizeof(DevClock) * B->nprob, cudaMemcpyDeviceToDevice,
                        B->stream);
    if (e != cudaSuccess && rc == AST_OK) rc = cuda_fail(e, "autotune clock restore");
    e = cudaStreamSynchronize(B->stream);
    if (e != cudaSuccess && rc == AST_OK) rc = cuda_fail(e, "autotune");
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    drop_graph(B);
    return rc;
}

}  // extern "C"
