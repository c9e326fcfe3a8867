// batch.cu -- many independent problems advanced by one persistent launch
// per time step (no counterpart in the reference, which runs one problem
// per MPI job).
//
// Every problem keeps its own context (operator blocks, mass inverse, RHS,
// state, degree, dt); the batch flattens all (problem, polyhedron) pairs
// into one work list.  A persistent grid of CTAs pulls items from an atomic
// queue and runs the same per-polyhedron body as the single-problem kernel
// (step_body.cuh) with the degree of the item's problem, so results are
// bit-identical to stepping each context alone.  A 1-thread kernel after
// each step advances the step counter (which selects each problem's buffer
// parity and time-function value) and resets the queue; the loop is launched
// as CUDA graphs of 16 steps.  The grid size and the item order (largest
// cost first or problem-major) are picked by a timing autotuner whose choice
// is cached per batch signature.  The autotuner also picks the tile shape:
// the number of column slices S per degree (kBatchShapes).  Shape 0, the
// default before tuning, is the single-problem kernel's, so results are then
// bit-identical to stepping each context alone; the other shapes group the
// row's partial sums differently (deterministic, equal to rounding).  On the
// matrix-free path (mf.cu) the items are grouped by degree and each degree
// present gets its own persistent launch per step, so every degree runs
// with its own register and shared-memory budget.

#include <algorithm>
#include <cstdlib>
#include <filesystem>
#include <fstream>
#include <map>
#include <mutex>
#include <numeric>
#include <sstream>
#include <string>
#include <vector>

#include "step_body.cuh"

using namespace stepk;

size_t lymph_mf_batch_problem_bytes();
int lymph_mf_batch_ctas_per_sm(int p);
void lymph_mf_batch_problem(const lymph_ctx* c, int* status, void* out);
int lymph_mf_batch_step(cudaStream_t st, const int* grid, const void* probs, const int2* items, const int* off,
                        int* queue, const int64_t* step_idx, const double* gvals, int64_t g_stride, int* launched);

namespace {

constexpr int BATCH_THREADS = 320;   // the p = 4 shape; lower degrees leave lanes idle
constexpr int BATCH_MINB = 4;
constexpr int BATCH_QUEUES = 4;      // item counters: one per degree on the matrix-free path

struct BatchProblem {
    StepArgs a;        // per-problem pointers; u0/un/out are filled per step
    double* buf[2];
    int cur0;          // buffer parity of the problem when the run started
    int p;
};

// Tile shapes the autotuner chooses from: column slices S for p = 1..4
// (index 0 unused); every ND * S fits the CTA's 320 threads.
constexpr int BATCH_SHAPES = 3;
constexpr int kBatchShapes[BATCH_SHAPES][5] = {{0, 8, 8, 4, 3}, {0, 16, 10, 5, 3}, {0, 24, 10, 5, 2}};

constexpr size_t zmax(size_t a, size_t b) { return a > b ? a : b; }
template <typename KT, int V> struct ShapeSmem {
    static constexpr size_t bytes =
        zmax(zmax(SmemSize<1, KT, kBatchShapes[V][1]>::bytes, SmemSize<2, KT, kBatchShapes[V][2]>::bytes),
             zmax(SmemSize<3, KT, kBatchShapes[V][3]>::bytes, SmemSize<4, KT, kBatchShapes[V][4]>::bytes));
};
template <typename KT> struct BatchSmem {
    static constexpr size_t bytes = zmax(ShapeSmem<KT, 0>::bytes, zmax(ShapeSmem<KT, 1>::bytes, ShapeSmem<KT, 2>::bytes));
};
static_assert(Deg<1>::ND * kBatchShapes[2][1] <= BATCH_THREADS && Deg<2>::ND * kBatchShapes[1][2] <= BATCH_THREADS &&
                  Deg<3>::ND * kBatchShapes[1][3] <= BATCH_THREADS && Deg<4>::ND * kBatchShapes[0][4] <= BATCH_THREADS,
              "every tile shape fits the CTA");

template <typename KT, int V>
__global__ void __launch_bounds__(BATCH_THREADS, BATCH_MINB)
k_step_batch(const BatchProblem* __restrict__ probs, const int2* __restrict__ items, int n_items, int* queue,
             const int64_t* step_idx, const double* gvals, int64_t g_stride) {
    __shared__ __align__(16) char smem[BatchSmem<KT>::bytes];
    __shared__ int s_item;
    const int64_t k = *step_idx;
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(queue, 1);
        __syncthreads();
        const int it = s_item;
        __syncthreads();
        if (it >= n_items) break;
        const int2 w = items[it];
        StepArgs A = probs[w.x].a;
        const int cur = probs[w.x].cur0 ^ (int)(k & 1);
        A.un = probs[w.x].buf[cur];
        A.u0 = probs[w.x].buf[cur ^ 1];
        A.out = probs[w.x].buf[cur ^ 1];
        A.gvals = gvals + (int64_t)w.x * g_stride;
        A.step_idx = step_idx;
        switch (probs[w.x].p) {
            case 1: step_poly<1, KT, MODE_STEP, kBatchShapes[V][1]>(A, w.y, smem); break;
            case 2: step_poly<2, KT, MODE_STEP, kBatchShapes[V][2]>(A, w.y, smem); break;
            case 3: step_poly<3, KT, MODE_STEP, kBatchShapes[V][3]>(A, w.y, smem); break;
            default: step_poly<4, KT, MODE_STEP, kBatchShapes[V][4]>(A, w.y, smem); break;
        }
    }
}

__global__ void k_batch_bump(int64_t* idx, int* queue) {
    *idx += 1;
    for (int i = 0; i < BATCH_QUEUES; ++i) queue[i] = 0;
}

std::string tune_cache_path() {
    const char* e = std::getenv("LYMPH_TUNE_CACHE");
    if (e && *e) return e;
    const char* h = std::getenv("HOME");
    return std::string(h ? h : "/tmp") + "/.cache/lymph3d_gb300_tune2.txt";
}

std::mutex g_tune_mu;

bool tune_lookup(const std::string& key, int* grid, int* order, int* shape) {
    std::lock_guard<std::mutex> l(g_tune_mu);
    std::ifstream f(tune_cache_path());
    std::string k;
    int g, o, sh;
    while (f >> k >> g >> o >> sh)
        if (k == key && sh >= 0 && sh < BATCH_SHAPES) { *grid = g; *order = o; *shape = sh; return true; }
    return false;
}

void tune_store(const std::string& key, int grid, int order, int shape) {
    std::lock_guard<std::mutex> l(g_tune_mu);
    std::string path = tune_cache_path();
    size_t slash = path.rfind('/');
    if (slash != std::string::npos && slash > 0) {
        std::error_code ec;  // the cache is optional: a directory that cannot be made skips the store
        std::filesystem::create_directories(path.substr(0, slash), ec);
        if (ec) return;
    }
    std::ofstream f(path, std::ios::app);
    f << key << " " << grid << " " << order << " " << shape << "\n";
}

}  // namespace

struct lymph_batch {
    std::vector<lymph_ctx*> ctx;
    int precision = LYMPH_FP64;
    cudaStream_t stream = nullptr;
    void* d_probs = nullptr;         // BatchProblem[n], or the matrix-free path's records
    int2* d_items = nullptr;
    int n_items = 0;
    std::vector<int2> items_lpt, items_natural;
    int order = 0;       // 0 = largest cost first, 1 = problem-major
    int grid = 0;
    int shape = 0;       // tile shape (kBatchShapes row) of the FP64 / FP32-block kernel
    int* d_queue = nullptr;          // BATCH_QUEUES item counters (one per degree on the matrix-free path)
    int mf_off[5] = {0, 0, 0, 0, 0};  // matrix-free path: degree p's items are [mf_off[p - 1], mf_off[p])
    int mf_occ[4] = {1, 1, 1, 1};     // matrix-free path: CTAs per SM of each degree's kernel
    int64_t* d_step_idx = nullptr;
    double* d_gvals = nullptr;
    int64_t gvals_cap = 0;
    int* d_status = nullptr;
    cudaGraphExec_t graph = nullptr;
    int graph_steps = 0;
    int64_t launches = 0;
    int step_nl = 2;     // kernels one batched step launches
    int sms = 0;
    std::string key;
};

namespace {

int upload_items(lymph_batch* b) {
    const std::vector<int2>& v0 = b->order == 0 ? b->items_lpt : b->items_natural;
    std::vector<int2> grouped;
    const std::vector<int2>* v = &v0;
    if (b->precision == LYMPH_MIXED_MF) {
        // one group per degree, each in the chosen order
        for (int p = 1; p <= 4; ++p) {
            b->mf_off[p - 1] = (int)grouped.size();
            for (const int2& w : v0)
                if (b->ctx[w.x]->p == p) grouped.push_back(w);
        }
        b->mf_off[4] = (int)grouped.size();
        v = &grouped;
    }
    LYMPH_CUDA_TRY(cudaMemcpyAsync(b->d_items, v->data(), v->size() * sizeof(int2), cudaMemcpyHostToDevice, b->stream));
    LYMPH_CUDA_TRY(cudaStreamSynchronize(b->stream));  // the host vector goes out of scope
    if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
    return LYMPH_OK;
}

int refresh_problems(lymph_batch* b) {
    if (b->precision == LYMPH_MIXED_MF) {
        const size_t rb = lymph_mf_batch_problem_bytes();
        std::vector<char> h(rb * b->ctx.size());
        for (size_t i = 0; i < b->ctx.size(); ++i) lymph_mf_batch_problem(b->ctx[i], b->d_status, h.data() + rb * i);
        LYMPH_CUDA_TRY(cudaMemcpyAsync(b->d_probs, h.data(), h.size(), cudaMemcpyHostToDevice, b->stream));
        return LYMPH_OK;
    }
    std::vector<BatchProblem> h(b->ctx.size());
    for (size_t i = 0; i < b->ctx.size(); ++i) {
        lymph_ctx* c = b->ctx[i];
        BatchProblem& P = h[i];
        P = BatchProblem();
        P.a.row_ptr = c->d_row_ptr;
        P.a.col = c->d_col;
        P.a.K = c->d_K;
        P.a.Minv = c->d_Minv;
        P.a.rhs_stat = c->d_rhs_stat;
        P.a.rhs_dyn = c->d_rhs_dyn;
        P.a.partial = nullptr;
        P.a.abs_idx = c->n_abs > 0 ? c->d_abs_idx : nullptr;
        P.a.Dabs = c->d_Dabs;
        P.a.Winv = c->d_Winv;
        P.a.dt = c->dt;
        P.a.status = b->d_status;
        P.a.n_poly = c->n_poly;
        P.buf[0] = c->d_buf[0];
        P.buf[1] = c->d_buf[1];
        P.cur0 = c->cur;
        P.p = c->p;
    }
    LYMPH_CUDA_TRY(cudaMemcpyAsync(b->d_probs, h.data(), h.size() * sizeof(BatchProblem), cudaMemcpyHostToDevice, b->stream));
    return LYMPH_OK;
}

template <typename KT>
void launch_shape(lymph_batch* b, const BatchProblem* probs, int64_t g_stride) {
    auto go = [&](auto kernel) {
        kernel<<<b->grid, BATCH_THREADS, 0, b->stream>>>(probs, b->d_items, b->n_items, b->d_queue, b->d_step_idx,
                                                         b->d_gvals, g_stride);
    };
    switch (b->shape) {
        case 1: go(k_step_batch<KT, 1>); break;
        case 2: go(k_step_batch<KT, 2>); break;
        default: go(k_step_batch<KT, 0>); break;
    }
}

int launch_step(lymph_batch* b, int64_t g_stride) {
    const BatchProblem* probs = (const BatchProblem*)b->d_probs;
    int nl = 1;
    if (b->precision == LYMPH_MIXED_MF) {
        // per degree: the tuned grid, at most what the SMs hold of that
        // degree's kernel and at most one CTA per item
        int grid[4];
        for (int p = 1; p <= 4; ++p) {
            const int n = b->mf_off[p] - b->mf_off[p - 1];
            grid[p - 1] = std::min(std::min(b->grid, b->mf_occ[p - 1] * b->sms), n);
        }
        LYMPH_TRY(lymph_mf_batch_step(b->stream, grid, b->d_probs, b->d_items, b->mf_off, b->d_queue, b->d_step_idx,
                                      b->d_gvals, g_stride, &nl));
    } else if (b->precision == LYMPH_MIXED) {
        launch_shape<float>(b, probs, g_stride);
    } else {
        launch_shape<double>(b, probs, g_stride);
    }
    k_batch_bump<<<1, 1, 0, b->stream>>>(b->d_step_idx, b->d_queue);
    b->step_nl = nl + 1;
    b->launches += b->step_nl;
    LYMPH_CUDA_TRY(cudaGetLastError());
    return LYMPH_OK;
}

// Runs n steps with the current grid/order; the time-function values are
// already on the device with stride g_stride per problem.
int run_loop(lymph_batch* b, int64_t n, int64_t g_stride, bool use_graph) {
    LYMPH_TRY(refresh_problems(b));
    LYMPH_CUDA_TRY(cudaMemsetAsync(b->d_step_idx, 0, sizeof(int64_t), b->stream));
    LYMPH_CUDA_TRY(cudaMemsetAsync(b->d_queue, 0, BATCH_QUEUES * sizeof(int), b->stream));
    const int R = 16;
    int64_t i = 0;
    if (use_graph && n >= R) {
        if (b->graph && b->graph_steps != (int)g_stride) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
        if (!b->graph) {
            cudaGraph_t g;
            LYMPH_CUDA_TRY(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
            int64_t l0 = b->launches;
            for (int j = 0; j < R; ++j) launch_step(b, g_stride);
            b->launches = l0;
            cudaError_t e = cudaStreamEndCapture(b->stream, &g);
            if (e != cudaSuccess) { lymph_set_error(std::string("batch graph capture: ") + cudaGetErrorString(e)); return LYMPH_ERR_CUDA; }
            e = cudaGraphInstantiate(&b->graph, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) { lymph_set_error(std::string("batch graph instantiate: ") + cudaGetErrorString(e)); return LYMPH_ERR_CUDA; }
            b->graph_steps = (int)g_stride;
        }
        for (; i + R <= n; i += R) {
            LYMPH_CUDA_TRY(cudaGraphLaunch(b->graph, b->stream));
            b->launches += (int64_t)b->step_nl * R;
        }
    }
    for (; i < n; ++i) LYMPH_TRY(launch_step(b, g_stride));
    // each problem's buffers flipped n times
    if (n & 1)
        for (lymph_ctx* c : b->ctx) c->cur ^= 1;
    return LYMPH_OK;
}

int upload_g(lymph_batch* b, const double* g, int64_t n_steps) {
    int64_t need = (int64_t)b->ctx.size() * n_steps;
    if (need > b->gvals_cap) {
        if (b->d_gvals) cudaFree(b->d_gvals);
        b->d_gvals = nullptr;
        b->gvals_cap = need;
        if (cudaMalloc(&b->d_gvals, sizeof(double) * (size_t)need) != cudaSuccess) {
            lymph_set_error("lymph_batch: cannot allocate the time-function table");
            return LYMPH_ERR_OOM;
        }
        if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
    }
    LYMPH_CUDA_TRY(cudaMemcpyAsync(b->d_gvals, g, sizeof(double) * (size_t)need, cudaMemcpyHostToDevice, b->stream));
    return LYMPH_OK;
}

int batch_status(lymph_batch* b, const char* where) {
    LYMPH_CUDA_TRY(cudaStreamSynchronize(b->stream));
    int st = 0;
    LYMPH_CUDA_TRY(cudaMemcpy(&st, b->d_status, sizeof(int), cudaMemcpyDeviceToHost));
    if (st) {
        LYMPH_CUDA_TRY(cudaMemset(b->d_status, 0, sizeof(int)));
        lymph_set_error(std::string(where) + ": non-finite value in a problem's state");
        return LYMPH_EXIT_INSTAB;
    }
    return LYMPH_OK;
}

}  // namespace

extern "C" {

int lymph_batch_create(lymph_ctx* const* ctxs, int32_t n, lymph_batch** out) {
    if (!out || !ctxs || n <= 0) { lymph_set_error("lymph_batch_create: bad argument"); return LYMPH_ERR_INVALID; }
    *out = nullptr;
    for (int i = 0; i < n; ++i) {
        if (!ctxs[i]) { lymph_set_error("lymph_batch_create: null context"); return LYMPH_ERR_INVALID; }
        if (!ctxs[i]->have_matrices) { lymph_set_error("lymph_batch_create: every context needs lymph_make_matrices first"); return LYMPH_ERR_ORDER; }
        if (ctxs[i]->precision != ctxs[0]->precision) { lymph_set_error("lymph_batch_create: mixed precisions in one batch"); return LYMPH_ERR_INVALID; }
    }
    lymph_batch* b = new lymph_batch();
    b->ctx.assign(ctxs, ctxs + n);
    b->precision = ctxs[0]->precision;
    auto fail = [&](int rc) { lymph_batch_destroy(b); return rc; };
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) { delete b; lymph_set_error("lymph_batch_create: stream"); return LYMPH_ERR_CUDA; }
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev);
    // work items and their cost (bytes of blocks streamed)
    std::vector<std::pair<int64_t, int2>> cost;
    std::ostringstream key;
    key << "sm" << b->sms << "_prec" << b->precision;
    std::map<int, int64_t> per_p;
    for (int i = 0; i < n; ++i) {
        lymph_ctx* c = ctxs[i];
        for (int P = 0; P < c->n_poly; ++P) {
            int64_t nb = c->h_row_ptr[P + 1] - c->h_row_ptr[P];
            cost.push_back({nb * (int64_t)c->nd * c->nd, make_int2(i, P)});
            b->items_natural.push_back(make_int2(i, P));
        }
        per_p[c->p] += c->n_blocks;
    }
    for (auto& kv : per_p) key << "_p" << kv.first << "b" << kv.second;
    b->key = key.str();
    std::stable_sort(cost.begin(), cost.end(), [](const std::pair<int64_t, int2>& x, const std::pair<int64_t, int2>& y) { return x.first > y.first; });
    for (auto& c : cost) b->items_lpt.push_back(c.second);
    b->n_items = (int)b->items_natural.size();
    const size_t prob_bytes = b->precision == LYMPH_MIXED_MF ? lymph_mf_batch_problem_bytes() : sizeof(BatchProblem);
    if (cudaMalloc(&b->d_probs, prob_bytes * n) != cudaSuccess ||
        cudaMalloc(&b->d_items, sizeof(int2) * b->n_items) != cudaSuccess ||
        cudaMalloc(&b->d_queue, BATCH_QUEUES * sizeof(int)) != cudaSuccess || cudaMalloc(&b->d_step_idx, sizeof(int64_t)) != cudaSuccess ||
        cudaMalloc(&b->d_status, sizeof(int)) != cudaSuccess) {
        lymph_set_error("lymph_batch_create: device allocation failed");
        return fail(LYMPH_ERR_OOM);
    }
    cudaMemsetAsync(b->d_status, 0, sizeof(int), b->stream);
    if (b->precision == LYMPH_MIXED_MF)
        for (int p = 1; p <= 4; ++p) b->mf_occ[p - 1] = lymph_mf_batch_ctas_per_sm(p);
    b->grid = 4 * b->sms;
    b->order = 0;
    b->shape = 0;
    int g, o, sh;
    if (tune_lookup(b->key, &g, &o, &sh)) { b->grid = g; b->order = o; b->shape = sh; }
    int rc = upload_items(b);
    if (rc) return fail(rc);
    *out = b;
    return LYMPH_OK;
}

int lymph_batch_destroy(lymph_batch* b) {
    if (!b) return LYMPH_OK;
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    for (void* p : {(void*)b->d_probs, (void*)b->d_items, (void*)b->d_queue, (void*)b->d_step_idx, (void*)b->d_gvals,
                    (void*)b->d_status})
        if (p) cudaFree(p);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return LYMPH_OK;
}

int lymph_batch_run(lymph_batch* b, int64_t n_steps, const double* gvals, float* ms_total) {
    NvtxRange nvtx_("lymph_batch_run");
    if (!b || n_steps < 0 || (n_steps > 0 && !gvals)) return LYMPH_ERR_INVALID;
    if (ms_total) *ms_total = 0.0f;
    if (n_steps == 0) return LYMPH_OK;
    for (lymph_ctx* c : b->ctx) cudaStreamSynchronize(c->stream);  // contexts' own work first
    LYMPH_TRY(upload_g(b, gvals, n_steps));
    cudaEvent_t e0, e1;
    LYMPH_CUDA_TRY(cudaEventCreate(&e0));
    LYMPH_CUDA_TRY(cudaEventCreate(&e1));
    cudaEventRecord(e0, b->stream);
    int rc = run_loop(b, n_steps, n_steps, true);
    cudaEventRecord(e1, b->stream);
    cudaEventSynchronize(e1);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms_total) *ms_total = ms;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    LYMPH_TRY(rc);
    return batch_status(b, "lymph_batch_run");
}

int lymph_batch_autotune(lymph_batch* b, int32_t trial_steps, int32_t use_cache, int32_t* grid, int32_t* order) {
    if (!b || trial_steps < 1) return LYMPH_ERR_INVALID;
    int g0, o0, s0;
    if (use_cache && tune_lookup(b->key, &g0, &o0, &s0)) {
        b->grid = g0;
        b->order = o0;
        b->shape = s0;
        LYMPH_TRY(upload_items(b));
    } else {
        // candidates: persistent grids of 1..k CTAs per SM (k: what one SM
        // holds of the step kernel), two item orders and, for the block
        // kernel, the tile shapes.  The trial steps advance the real state, so the state
        // is saved and restored around the trials.
        std::vector<std::vector<double>> save(b->ctx.size() * 2);
        for (size_t i = 0; i < b->ctx.size(); ++i) {
            lymph_ctx* c = b->ctx[i];
            size_t nv = (size_t)c->n_poly * c->nd;
            for (int k = 0; k < 2; ++k) {
                save[2 * i + k].resize(nv);
                LYMPH_CUDA_TRY(cudaMemcpy(save[2 * i + k].data(), c->d_buf[k], nv * sizeof(double), cudaMemcpyDeviceToHost));
            }
        }
        std::vector<int> curs;
        for (lymph_ctx* c : b->ctx) curs.push_back(c->cur);
        std::vector<double> g((size_t)b->ctx.size() * (trial_steps + 1), 0.0);
        LYMPH_TRY(upload_g(b, g.data(), trial_steps + 1));
        float best = 1e30f;
        int bg = b->grid, bo = b->order, bs = b->shape;
        const int n_shapes = b->precision == LYMPH_MIXED_MF ? 1 : BATCH_SHAPES;
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        const int max_mult =
            b->precision == LYMPH_MIXED_MF ? *std::max_element(b->mf_occ, b->mf_occ + 4) : BATCH_MINB;
        for (int shp = 0; shp < n_shapes; ++shp)
        for (int ord = 0; ord < 2; ++ord)
            for (int mult = 1; mult <= max_mult; ++mult) {
                b->shape = shp;
                b->order = ord;
                b->grid = mult * b->sms;
                LYMPH_TRY(upload_items(b));
                LYMPH_TRY(run_loop(b, 1, trial_steps + 1, false));  // warm-up
                cudaEventRecord(e0, b->stream);
                LYMPH_TRY(run_loop(b, trial_steps, trial_steps + 1, false));
                cudaEventRecord(e1, b->stream);
                cudaEventSynchronize(e1);
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, e0, e1);
                if (ms < best) { best = ms; bg = b->grid; bo = ord; bs = shp; }
            }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        for (size_t i = 0; i < b->ctx.size(); ++i) {
            lymph_ctx* c = b->ctx[i];
            size_t nv = (size_t)c->n_poly * c->nd;
            for (int k = 0; k < 2; ++k)
                LYMPH_CUDA_TRY(cudaMemcpy(c->d_buf[k], save[2 * i + k].data(), nv * sizeof(double), cudaMemcpyHostToDevice));
            c->cur = curs[i];
        }
        LYMPH_CUDA_TRY(cudaMemset(b->d_status, 0, sizeof(int)));
        b->grid = bg;
        b->order = bo;
        b->shape = bs;
        LYMPH_TRY(upload_items(b));
        tune_store(b->key, bg, bo, bs);
    }
    if (grid) *grid = b->grid;
    if (order) *order = b->order;
    LYMPH_CUDA_TRY(cudaStreamSynchronize(b->stream));
    return LYMPH_OK;
}

int lymph_batch_schedule(const lymph_batch* b, int32_t* grid, int32_t* order, int32_t* shape) {
    if (!b) return LYMPH_ERR_INVALID;
    if (grid) *grid = b->grid;
    if (order) *order = b->order;
    if (shape) *shape = b->shape;
    return LYMPH_OK;
}

int lymph_batch_launch_count(const lymph_batch* b, int64_t* count) {
    if (!b || !count) return LYMPH_ERR_INVALID;
    *count = b->launches;
    return LYMPH_OK;
}

}  // extern "C"
