// C ABI of the TGV-DCT path (include/tgvdct.h): contexts, status codes, the
// iteration loop with its callback, and the host-buffer drop-in launchers.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "common.cuh"

namespace tgvdct {
namespace {
thread_local std::string g_last_error;
}
void set_error(const std::string& msg) { g_last_error = msg; }
}  // namespace tgvdct

using namespace tgvdct;

struct tgvdct_context {
    tgvdct_params prm;
    TgvState st;
    void* state_block = nullptr;
    DctPlan* plan = nullptr;
    uint32_t iterations_run = 0;
    uint64_t loop_launches = 0;  // iteration kernels the last loop launched
    // stopping: a request from any thread, and the energy checks of the last loop
    std::atomic<bool> stop_requested{false};
    double* energy_dev = nullptr;  // 3 sums of one energy evaluation
    std::vector<double> energy_history;
    // pinned host buffers for callbacks that receive host copies
    float* host_cb = nullptr;
    size_t host_cb_count = 0;
    // device scratch for the per-callback deshade of tgvdct_process_dev
    float* cb_dev = nullptr;
    // masked deshade: the caller's mask (weights of the epilogue) and the domain
    // derived from it (voxels with mask >= 1 are iterated)
    float* domain_mask = nullptr;
    uint8_t* domain = nullptr;
    uint32_t* tile_flags = nullptr;  // per-block plane ranges of the fused TMA kernel
    // CUDA graphs of loop stretches, captured on a private stream and replayed on the
    // caller's.  Each is valid for its length, starting parity, step, domain and
    // z-chunk; a few are kept (least recently used goes first).
    struct LoopGraph {
        cudaGraphExec_t exec = nullptr;
        uint32_t len = 0;
        int cur = -1, end_cur = -1, zchunk = 0, launches = 0;
        TgvStep step{};
        const void* domain = nullptr;
        uint64_t used = 0;
    };
    LoopGraph graphs[4];
    uint64_t graph_clock = 0;
    cudaStream_t capture_stream = nullptr;
    // reverse mode: checkpoints of the last checkpointed forward run, the states of
    // one recomputed segment, and the adjoint state with its scratch fields
    void* ckpt_block = nullptr;
    size_t ckpt_bytes = 0;
    uint32_t ckpt_every = 0, ckpt_K = 0, ckpt_count = 0;
    bool have_ckpt = false;
    void* seg_block = nullptr;
    size_t seg_bytes = 0;
    void* adj_block = nullptr;
    size_t adj_bytes = 0;
    std::shared_ptr<void> step_cache;  // tensor maps of the recompute steps
    // the whole backward pass as one CUDA graph, valid while its key holds
    cudaGraphExec_t bwd_graph = nullptr;
    struct BwdKey {
        const void *ckpt = nullptr, *seg = nullptr, *adj = nullptr;
        uint32_t every = 0, K = 0, count = 0;
        int zchunk = 0;
        int passes = 0;  // AdjointPasses
        TgvStep step{};
    } bwd_key;
};

namespace {

size_t voxels(const tgvdct_params& p) { return (size_t)p.width * p.height * p.depth; }

void validate(const tgvdct_params* p) {
    TGV_REQUIRE(p != nullptr, "null parameter block");
    TGV_REQUIRE(p->width >= 1 && p->height >= 1 && p->depth >= 1, "width, height, depth must be >= 1");
    TGV_REQUIRE(p->depth <= 65535, "depth must be <= 65535");
    TGV_REQUIRE((uint64_t)p->width * p->height * p->depth <= (uint64_t)1 << 34,
                "volume larger than 2^34 voxels");
    TGV_REQUIRE(p->geometry == TGVDCT_GEOMETRY_3D || p->geometry == TGVDCT_GEOMETRY_2D,
                "unknown geometry");
    TGV_REQUIRE(p->geometry == TGVDCT_GEOMETRY_3D || p->depth == 1,
                "2-D geometry requires depth == 1");
    TGV_REQUIRE(p->data_term == TGVDCT_DATA_L1 || p->data_term == TGVDCT_DATA_L2,
                "unknown data term");
    TGV_REQUIRE(p->state_precision >= TGVDCT_STATE_FP32 &&
                    p->state_precision <= TGVDCT_STATE_FX16_DUAL,
                "unknown state precision");
    TGV_REQUIRE(p->dct_mode >= TGVDCT_DCT_FP32 && p->dct_mode <= TGVDCT_DCT_BF16X3,
                "unknown DCT mode");
    TGV_REQUIRE(p->poisson_eigen == TGVDCT_EIGEN_REFERENCE ||
                    p->poisson_eigen == TGVDCT_EIGEN_ACCURATE,
                "unknown Poisson eigenvalue mode");
    TGV_REQUIRE(std::isfinite(p->alpha0) && p->alpha0 > 0.f, "alpha0 must be > 0");
    TGV_REQUIRE(std::isfinite(p->alpha1) && p->alpha1 > 0.f, "alpha1 must be > 0");
    TGV_REQUIRE(std::isfinite(p->lambda) && p->lambda >= 0.f, "lambda must be >= 0");
    TGV_REQUIRE(std::isfinite(p->tau) && p->tau > 0.f, "tau must be > 0");
    TGV_REQUIRE(std::isfinite(p->sigma) && p->sigma > 0.f, "sigma must be > 0");
    TGV_REQUIRE(std::isfinite(p->theta), "theta must be finite");
    TGV_REQUIRE(p->iteration_kernel >= TGVDCT_KERNEL_AUTO &&
                    p->iteration_kernel <= TGVDCT_KERNEL_FUSED_SHIFTED,
                "unknown iteration kernel");
    TGV_REQUIRE(p->z_chunk >= 0, "z_chunk must be >= 0");
    TGV_REQUIRE(p->energy_tolerance >= 0.f && std::isfinite(p->energy_tolerance),
                "energy_tolerance must be finite and >= 0");
}

// The automatic choice: shifted passes for volumes (runs of iterations as the primal
// step of one and the dual step of the next, 108 bytes per voxel-iteration; single
// iterations and the states they do not take run as the fused z-marching pass: at
// 256 x 256 x 192 0.258 against 0.289 ms per iteration); the two-pass kernels for a
// single plane, where the fused pass has no planes to pipeline (at 512^2, 1024^2 and
// 2048^2 the two passes take 6.2, 15.5 and 87 ms per 1000 iterations against 11.0,
// 39.8 and 164 ms).  Every kernel gives the same bits.
int kernel_of(const tgvdct_params& p) {
    switch (p.iteration_kernel) {
        case TGVDCT_KERNEL_TWO_PASS: return TGV_KERNEL_TWO_PASS;
        case TGVDCT_KERNEL_FUSED_REGISTER: return TGV_KERNEL_FUSED_REGISTER;
        case TGVDCT_KERNEL_FUSED: return TGV_KERNEL_FUSED;
        case TGVDCT_KERNEL_FUSED_SHIFTED: return TGV_KERNEL_SHIFTED;
        default: return p.depth == 1 ? TGV_KERNEL_TWO_PASS : TGV_KERNEL_SHIFTED;
    }
}

// Planes per block of the fused kernel.  The blocks of one launch run in waves of
// (SMs x 2) resident blocks, so a launch whose block count ends just short of a full
// wave leaves the GPU part-empty at its end; each z-chunk also pays a prologue of
// about 0.7 planes.  Over balanced chunk counts k (z = ceil(D / k), 12 <= z <= 64)
// this picks the best (wave fill) x (1 - 0.7 / z).  At 256 x 256 x 192 on 152 SMs:
// k = 7, z = 28, 1792 blocks = 5.89 waves (measured 333.8 us per iteration, against
// 338 us at z = 24 and 353 us at z = 32).
int auto_zchunk(const tgvdct_params& p) {
    if (p.z_chunk > 0) return (int)p.z_chunk;
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        sms = 152;
    }
    const double slots = 2.0 * sms;
    const double tiles = (double)((p.width + 31) / 32) * ((p.height + 7) / 8);
    const long long D = p.depth;
    int best_z = (int)std::min<long long>(D, 64);
    double best = -1.0;
    for (long long k = 1; k <= D; ++k) {
        const long long z = (D + k - 1) / k;
        if (z > 64) continue;
        if (z < 12 && best >= 0.0) break;
        const double waves = tiles * (double)k / slots;
        const double fill = waves / std::ceil(waves);
        const double score = fill * (1.0 - 0.7 / (double)z);
        if (score > best + 1e-12) {
            best = score;
            best_z = (int)z;
        }
    }
    return best_z;
}

// Planes per block when a domain mask is set.  The blocks' plane ranges are trimmed to
// the domain and so differ in length; a grid of at most one wave keeps every block
// resident at once and the longest one sets the time, so it takes half the chunk.  At
// 128 x 128 x 96 with an ellipsoid domain: 55.6 -> 40.4 us per iteration (24 -> 12
// planes); at 256 x 256 x 192 the unmasked choice stays the fastest.
int masked_zchunk(const tgvdct_params& p) {
    const int z = auto_zchunk(p);
    if (p.z_chunk > 0) return z;
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        sms = 152;
    }
    const long long blocks = (long long)((p.width + 31) / 32) * ((p.height + 7) / 8) *
                             (((long long)p.depth + z - 1) / z);
    return blocks <= 2LL * sms ? std::max(1, (z + 1) / 2) : z;
}

void check_device() {
    int dev = 0, n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        set_error("no CUDA device available");
        throw Error{TGVDCT_ERR_NO_DEVICE};
    }
    TGV_CUDA(cudaGetDevice(&dev));
    int major = 0, minor = 0;
    TGV_CUDA(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
    TGV_CUDA(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev));
    if (major != 10 || minor != 3) {
        set_error("this library is built for sm_103a (GB300); device is sm_" +
                  std::to_string(major) + std::to_string(minor));
        throw Error{TGVDCT_ERR_NO_DEVICE};
    }
}

TgvStep step_of(const tgvdct_params& p) {
    TgvStep k;
    k.tau = p.tau;
    k.sigma = p.sigma;
    k.theta = p.theta;
    k.lambda = p.lambda;
    k.alpha0 = p.alpha0;
    k.alpha1 = p.alpha1;
    k.data_term = p.data_term;
    return k;
}

template <class F>
tgvdct_status guarded(F&& f) {
    try {
        return f();
    } catch (const Error& e) {
        return e.status;
    } catch (const std::bad_alloc&) {
        set_error("host allocation failed");
        return TGVDCT_ERR_OOM;
    } catch (...) {
        set_error("unexpected exception");
        return TGVDCT_ERR_CUDA;
    }
}

DctPlan* plan_of(tgvdct_context* c) {
    if (!c->plan) {
        c->plan = dct_plan_create((int)c->prm.width, (int)c->prm.height, (int)c->prm.depth);
        c->plan->wait_ns = c->st.wait_ns;
    }
    return c->plan;
}

float* host_cb_buffers(tgvdct_context* c) {
    const size_t need = 4 * voxels(c->prm);
    if (c->host_cb_count < need) {
        if (c->host_cb) cudaFreeHost(c->host_cb);
        c->host_cb = nullptr;
        c->host_cb_count = 0;
        TGV_CUDA(cudaMallocHost(&c->host_cb, need * sizeof(float)));
        c->host_cb_count = need;
    }
    return c->host_cb;
}

// Hands u, a, b, c (device) to a callback: host copies unless callback_on_device.
int deliver(tgvdct_context* c, tgvdct_iteration_callback cb, void* user, uint32_t it,
            const float* u, const float* a, const float* b, const float* cc, cudaStream_t s) {
    const size_t n = voxels(c->prm);
    if (c->prm.callback_on_device) {
        TGV_CUDA(cudaStreamSynchronize(s));
        return cb(it, c->prm.iteration_count, u, a, b, cc, user);
    }
    float* h = host_cb_buffers(c);
    const float* src[4] = {u, a, b, cc};
    const float* dst[4] = {nullptr, nullptr, nullptr, nullptr};
    for (int k = 0; k < 4; ++k) {
        if (!src[k]) continue;
        TGV_CUDA(cudaMemcpyAsync(h + k * n, src[k], n * 4, cudaMemcpyDeviceToHost, s));
        dst[k] = h + k * n;
    }
    TGV_CUDA(cudaStreamSynchronize(s));
    return cb(it, c->prm.iteration_count, dst[0], dst[1], dst[2], dst[3], user);
}

// Stretches of at least kMinGraphRun iterations run as CUDA graph replays of at most
// kMaxGraphRun iterations (a stop request is honoured between replays).  Longer
// replays also mean fewer runs of shifted passes, each of which pays one dual and one
// primal step of the two-pass kernels.
constexpr uint32_t kMinGraphRun = 16, kMaxGraphRun = 512;

bool same_step(const TgvStep& a, const TgvStep& b) {
    return a.tau == b.tau && a.sigma == b.sigma && a.theta == b.theta && a.lambda == b.lambda &&
           a.alpha0 == b.alpha0 && a.alpha1 == b.alpha1 && a.data_term == b.data_term;
}

void drop_loop_graphs(tgvdct_context* c) {
    for (auto& g : c->graphs) {
        if (g.exec) cudaGraphExecDestroy(g.exec);
        g = tgvdct_context::LoopGraph();
    }
}

// The graph of `len` iterations from the state's current parity with step k, built on
// first use (every kernel attribute is set before the capture; the capture runs
// nothing, so the state's parity is put back).  Null when capture is not possible.
tgvdct_context::LoopGraph* loop_graph(tgvdct_context* c, const TgvStep& k, uint32_t len) {
    for (auto& g : c->graphs)
        if (g.exec && g.len == len && same_step(g.step, k) && g.domain == c->st.domain &&
            g.cur == c->st.cur && g.zchunk == c->st.zchunk) {
            g.used = ++c->graph_clock;
            return &g;
        }
    tgvdct_context::LoopGraph* slot = &c->graphs[0];
    for (auto& g : c->graphs)
        if (!g.exec || (slot->exec && g.used < slot->used)) slot = &g;
    if (slot->exec) cudaGraphExecDestroy(slot->exec);
    *slot = tgvdct_context::LoopGraph();
    if (!c->capture_stream &&
        cudaStreamCreateWithFlags(&c->capture_stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    cudaGraph_t g = nullptr;
    tgv_prepare_launches(c->st);
    if (cudaStreamBeginCapture(c->capture_stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    const int cur = c->st.cur;
    const int launches = tgv_iterate_n(c->st, k, len, c->capture_stream);
    const int end_cur = c->st.cur;
    c->st.cur = cur;
    const cudaError_t e = cudaStreamEndCapture(c->capture_stream, &g);
    if (e != cudaSuccess || !g) {
        cudaGetLastError();
        return nullptr;
    }
    const cudaError_t ie = cudaGraphInstantiate(&slot->exec, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) {
        cudaGetLastError();
        slot->exec = nullptr;
        return nullptr;
    }
    slot->len = len;
    slot->cur = cur;
    slot->end_cur = end_cur;
    slot->zchunk = c->st.zchunk;
    slot->launches = launches;
    slot->step = k;
    slot->domain = c->st.domain;
    slot->used = ++c->graph_clock;
    return slot;
}

// The weighted primal energy of the loop's current (u, v) (synchronous).
double state_energy(tgvdct_context* c, cudaStream_t s) {
    if (!c->energy_dev) TGV_CUDA(cudaMalloc(&c->energy_dev, 3 * sizeof(double)));
    const auto& p = c->prm;
    tgv_energy_terms(c->st.f, c->st.u, c->st.v[0], c->st.v[1], c->st.v[2], (int)p.width,
                     (int)p.height, (int)p.depth, c->st.three, p.data_term, c->energy_dev, s);
    double h[3];
    TGV_CUDA(cudaMemcpyAsync(h, c->energy_dev, sizeof(h), cudaMemcpyDeviceToHost, s));
    TGV_CUDA(cudaStreamSynchronize(s));
    return (double)p.lambda * h[0] + (double)p.alpha1 * h[1] + (double)p.alpha0 * h[2];
}

// The iteration loop on the context's state (st.f already holds the input).
// `on_iteration` decides what a callback sees; returns true if stopped.  The host
// looks at the state only after iterations j > 0 with j % paint == 0 (callbacks,
// tgv2_common.cu:381-384) or j % check == 0 (energy checks): the iterations up to
// the next such j run as one stretch (tgv_iterate_n, shifted passes where the state
// allows), as CUDA graph replays of up to kMaxGraphRun iterations where it has at
// least kMinGraphRun (the small-volume loops are launch-bound otherwise).  A stop
// request is honoured between stretches and graph replays; the energy test after its
// checks.
template <class OnIteration>
bool run_loop(tgvdct_context* c, cudaStream_t s, bool have_cb, OnIteration&& on_iteration,
              bool from_initial_state = true) {
    NvtxRange range("tgvdct loop");
    const TgvStep k = step_of(c->prm);
    if (from_initial_state) tgv_state_init(c->st, s);
    const uint32_t n_it = c->prm.iteration_count, paint = c->prm.paint_iteration_interval;
    const uint32_t check = c->prm.energy_check_interval;
    const double tol = c->prm.energy_tolerance;
    const bool cb_on = have_cb && paint > 0;
    auto next_multiple = [](uint32_t it, uint32_t m) {
        return (it % m == 0) ? it : (it / m + 1) * m;
    };
    c->iterations_run = 0;
    c->loop_launches = 0;
    c->energy_history.clear();
    tgv_prepare_launches(c->st);
    for (uint32_t it = 0; it < n_it;) {
        if (c->stop_requested.exchange(false)) {
            c->iterations_run = it;
            return true;
        }
        // the last iteration of this stretch: the next one the host looks after
        uint32_t last = n_it - 1;
        const uint32_t from = std::max<uint32_t>(it, 1);
        if (cb_on) last = std::min(last, next_multiple(from, paint));
        if (check > 0) last = std::min(last, next_multiple(from, check));
        uint32_t run = last + 1 - it;
        bool stopped = false;
        // graph replays; not at the loop's first iteration, so that a short loop never
        // pays a capture
        while (it > 0 && run >= kMinGraphRun) {
            const uint32_t len = std::min(run, kMaxGraphRun);
            tgvdct_context::LoopGraph* g = loop_graph(c, k, len);
            if (!g) break;
            TGV_CUDA(cudaGraphLaunch(g->exec, s));
            c->st.cur = g->end_cur;
            c->loop_launches += (uint64_t)g->launches;
            it += len;
            run -= len;
            if (run > 0 && c->stop_requested.exchange(false)) {
                stopped = true;
                break;
            }
        }
        if (stopped) {
            c->iterations_run = it;
            return true;
        }
        if (it == 0 && run > kMinGraphRun) run = 1;  // the first iteration alone, then graphs
        if (run > 0) {
            c->loop_launches += (uint64_t)tgv_iterate_n(c->st, k, run, s);
            it += run;
        }
        const uint32_t j = it - 1;  // the last iteration run
        if (j != last) continue;
        if (cb_on && j > 0 && j % paint == 0) {
            if (on_iteration(j)) {
                c->iterations_run = j + 1;
                return true;
            }
        }
        if (check > 0 && j > 0 && j % check == 0) {
            const double e = state_energy(c, s);
            const bool settled = tol > 0.0 && !c->energy_history.empty() &&
                                 std::fabs(e - c->energy_history.back()) <= tol * std::fabs(e);
            c->energy_history.push_back(e);
            if (settled) {
                c->iterations_run = j + 1;
                return true;
            }
        }
    }
    c->iterations_run = n_it;
    return false;
}

// Reads and clears the TGV kernels' device error flag (a pipeline wait timed out).
void check_tgv_flag(tgvdct_context* c, cudaStream_t s) {
    if (!c->st.err) return;
    int h = 0;
    TGV_CUDA(cudaMemcpyAsync(&h, c->st.err, sizeof(int), cudaMemcpyDeviceToHost, s));
    TGV_CUDA(cudaStreamSynchronize(s));
    if (h) {
        TGV_CUDA(cudaMemsetAsync(c->st.err, 0, sizeof(int), s));
        set_error("a TGV iteration kernel timed out waiting on its load pipeline");
        throw Error{TGVDCT_ERR_TIMEOUT};
    }
}

void create_into(const tgvdct_params* p, tgvdct_context** out) {
    validate(p);
    TGV_REQUIRE(out != nullptr, "null context output pointer");
    check_device();
    tgvdct_context* c = new tgvdct_context();
    c->prm = *p;
    c->st.W = (int)p->width;
    c->st.H = (int)p->height;
    c->st.D = (int)p->depth;
    c->st.three = p->geometry == TGVDCT_GEOMETRY_3D;
    c->st.precision = p->state_precision;
    c->st.kernel = kernel_of(*p);
    c->st.zchunk = auto_zchunk(*p);
    const size_t bytes = tgv_state_bytes(c->st.W, c->st.H, c->st.D, c->st.three, c->st.precision,
                                         c->st.kernel);
    cudaError_t e = cudaMalloc(&c->state_block, bytes);
    if (e != cudaSuccess) {
        delete c;
        cudaGetLastError();
        set_error(std::string("cudaMalloc of the TGV state: ") + cudaGetErrorString(e));
        throw Error{TGVDCT_ERR_OOM};
    }
    tgv_state_bind(c->st, (char*)c->state_block);
    *out = c;
}

void destroy_ctx(tgvdct_context* c) {
    if (!c) return;
    if (c->ckpt_block) cudaFree(c->ckpt_block);
    if (c->seg_block) cudaFree(c->seg_block);
    if (c->adj_block) cudaFree(c->adj_block);
    if (c->state_block) cudaFree(c->state_block);
    if (c->cb_dev) cudaFree(c->cb_dev);
    if (c->domain_mask) cudaFree(c->domain_mask);
    if (c->domain) cudaFree(c->domain);
    if (c->tile_flags) cudaFree(c->tile_flags);
    if (c->host_cb) cudaFreeHost(c->host_cb);
    drop_loop_graphs(c);
    if (c->bwd_graph) cudaGraphExecDestroy(c->bwd_graph);
    if (c->energy_dev) cudaFree(c->energy_dev);
    if (c->capture_stream) cudaStreamDestroy(c->capture_stream);
    dct_plan_destroy(c->plan);
    delete c;
}

// (re)allocates a context-owned device block of at least `bytes`
// Grows *block to at least `bytes`; returns whether it was reallocated.
bool ensure_block(void** block, size_t* have, size_t bytes) {
    if (*have >= bytes && *block) return false;
    if (*block) cudaFree(*block);
    *block = nullptr;
    *have = 0;
    TGV_CUDA(cudaMalloc(block, bytes));
    *have = bytes;
    return true;
}

TgvFullDev full_state_at(void* block, size_t index, size_t n) {
    TgvFullDev d;
    tgv_full_state_bind(d, (char*)block + index * tgv_full_state_bytes(n), n);
    return d;
}

void require_reverse_mode(const tgvdct_context* c) {
    if (c->prm.state_precision != TGVDCT_STATE_FP32 || c->prm.geometry != TGVDCT_GEOMETRY_3D) {
        set_error("the reverse mode needs FP32 state and 3-D geometry");
        throw Error{TGVDCT_ERR_UNSUPPORTED};
    }
    if (c->domain) {
        set_error("the reverse mode does not support a domain mask");
        throw Error{TGVDCT_ERR_UNSUPPORTED};
    }
}

void set_domain(tgvdct_context* c, const float* mask_dev, cudaStream_t s) {
    const size_t n = voxels(c->prm);
    if (!mask_dev) {
        TGV_CUDA(cudaStreamSynchronize(s));
        if (c->domain_mask) TGV_CUDA(cudaFree(c->domain_mask));
        if (c->domain) TGV_CUDA(cudaFree(c->domain));
        if (c->tile_flags) TGV_CUDA(cudaFree(c->tile_flags));
        c->domain_mask = nullptr;
        c->domain = nullptr;
        c->tile_flags = nullptr;
        c->st.domain = nullptr;
        c->st.tile_active = nullptr;
        c->st.zchunk = auto_zchunk(c->prm);
        return;
    }
    if (!c->domain) {
        if (cudaMalloc(&c->domain_mask, n * 4) != cudaSuccess ||
            cudaMalloc(&c->domain, n) != cudaSuccess ||
            cudaMalloc(&c->tile_flags, tgv_tile_flags_bytes(c->st)) != cudaSuccess) {
            cudaGetLastError();
            if (c->domain_mask) cudaFree(c->domain_mask);
            if (c->domain) cudaFree(c->domain);
            c->domain_mask = nullptr;
            c->domain = nullptr;
            c->tile_flags = nullptr;
            set_error("device allocation of the domain mask failed");
            throw Error{TGVDCT_ERR_OOM};
        }
    }
    TGV_CUDA(cudaMemcpyAsync(c->domain_mask, mask_dev, n * 4, cudaMemcpyDeviceToDevice, s));
    build_domain(c->domain_mask, n, c->domain, s);
    c->st.domain = c->domain;
    c->st.zchunk = masked_zchunk(c->prm);
    tgv_build_tile_flags(c->st, c->tile_flags, s);
}

struct CtxGuard {
    tgvdct_context* c = nullptr;
    ~CtxGuard() { destroy_ctx(c); }
};

struct DevBuf {
    float* p = nullptr;
    explicit DevBuf(size_t n) {
        if (n) TGV_CUDA(cudaMalloc(&p, n * sizeof(float)));
    }
    ~DevBuf() {
        if (p) cudaFree(p);
    }
};

// ---- the host-buffer calls' context cache ---------------------------------------------
// The one-shot host-buffer calls (the reference's per-volume entry points) keep their
// last context and device buffers, so that a caller streaming volumes of one shape
// through them pays the state allocation, the DCT plan and the graph captures once
// (about 4 ms of a 446 ms deshade at 256 x 256 x 192). One entry, keyed by the
// parameters, the entry point and the device. A call that finds the entry held (by
// another thread, or by an outer call whose iteration callback re-entered the
// library) builds a private context; a call that fails drops the entry.
// tgvdct_release_cached frees it.
struct HostCache {
    std::atomic<bool> busy{false};
    tgvdct_context* c = nullptr;
    int kind = 0, dev = -1;
    float* bufs = nullptr;
    size_t bufs_floats = 0;
};
HostCache& host_cache() {
    static HostCache* h = new HostCache();  // never destroyed: no CUDA calls at exit
    return *h;
}
void host_cache_drop(HostCache& h) {
    destroy_ctx(h.c);
    h.c = nullptr;
    if (h.bufs) cudaFree(h.bufs);
    h.bufs = nullptr;
    h.bufs_floats = 0;
}

// The entry points that lease contexts (the cache key's `kind`).
enum HostKind {
    HK_PROCESS = 1,
    HK_PROCESS_MASKED,
    HK_DESHADE_LAUNCH,
    HK_DESHADE_MASKED_LAUNCH,
    HK_RUN,
    HK_DENOISE_LAUNCH,
};

// Exclusive use of the cache entry while it lives (when `owned`).
struct CacheClaim {
    bool owned = false;
    CacheClaim() {
        bool idle = false;
        owned = host_cache().busy.compare_exchange_strong(idle, true);
    }
    ~CacheClaim() {
        if (owned) host_cache().busy.store(false);
    }
    CacheClaim(const CacheClaim&) = delete;
    CacheClaim& operator=(const CacheClaim&) = delete;
};

// A context and `nbuf` device buffers of n floats for one host-buffer call: the
// cached entry when it is free, else a private context. commit() after a call that
// succeeded keeps the entry for the next call.
class HostLease {
  public:
    HostLease(const tgvdct_params& p, int kind, int nbuf) : n_(voxels(p)) {
        if (claim_.owned) {
            HostCache& h = host_cache();
            int dev = -1;
            TGV_CUDA(cudaGetDevice(&dev));
            if (h.c && (h.kind != kind || h.dev != dev ||
                        std::memcmp(&h.c->prm, &p, sizeof(tgvdct_params)) != 0))
                host_cache_drop(h);
            if (!h.c) {
                create_into(&p, &h.c);
                h.kind = kind;
                h.dev = dev;
            }
            const size_t want = (size_t)nbuf * n_;
            if (h.bufs_floats < want) {
                if (h.bufs) cudaFree(h.bufs);
                h.bufs = nullptr;
                h.bufs_floats = 0;
                TGV_CUDA(cudaMalloc(&h.bufs, want * sizeof(float)));
                h.bufs_floats = want;
            }
            c = h.c;
            bufs_ = h.bufs;
        } else {
            create_into(&p, &own_.c);
            c = own_.c;
            if (nbuf) {
                own_bufs_ = std::make_unique<DevBuf>((size_t)nbuf * n_);
                bufs_ = own_bufs_->p;
            }
        }
    }
    ~HostLease() {
        if (claim_.owned && !committed_) host_cache_drop(host_cache());
    }
    HostLease(const HostLease&) = delete;
    HostLease& operator=(const HostLease&) = delete;
    void commit() { committed_ = true; }
    float* buf(int k) const { return bufs_ + (size_t)k * n_; }
    tgvdct_context* c = nullptr;

  private:
    CacheClaim claim_;  // first: released after everything else
    size_t n_;
    CtxGuard own_;
    std::unique_ptr<DevBuf> own_bufs_;
    float* bufs_ = nullptr;
    bool committed_ = false;
};

void process_on_device(tgvdct_context* c, const float* f_dev, const float* mask_dev, bool clamp,
                       bool add_back, bool log_domain, float* u_dev, float* l_dev, float* r_dev,
                       tgvdct_iteration_callback cb, void* user, cudaStream_t s) {
    NvtxRange range("tgvdct deshade");
    const size_t n = voxels(c->prm);
    TGV_CUDA(cudaMemcpyAsync(c->st.f, f_dev, n * 4, cudaMemcpyDeviceToDevice, s));
    if (log_domain) log_inplace(c->st.f, n, s);
    DctPlan* plan = plan_of(c);
    // The masked processor weights l and r by its mask and, without the background
    // add-back, multiplies r by it once more (TGVDeshadeMaskedProcessor.cpp:186-211).
    const bool masked = c->domain != nullptr;
    if (masked) mask_dev = c->domain_mask;
    const bool mask_shading = mask_dev != nullptr;
    const bool stopped = run_loop(c, s, cb != nullptr, [&](uint32_t it) {
        // The GUI module deshades at every paint interval and hands u, l, r to its
        // callback (TGVDeshadeProcessor.cpp:241-261); here that runs on the device.
        if (!c->cb_dev) TGV_CUDA(cudaMalloc(&c->cb_dev, 2 * n * sizeof(float)));
        float* l = c->cb_dev;
        float* r = c->cb_dev + n;
        poisson_integrate(plan, c->st.v[0], c->st.v[1], c->st.three ? c->st.v[2] : nullptr, l,
                          c->prm.dct_mode, c->prm.poisson_eigen, s);
        deshade_epilogue(c->st.u, l, mask_dev, n, mask_shading, clamp, add_back, r, s, masked);
        return deliver(c, cb, user, it, c->st.u, l, r, nullptr, s) != 0;
    });
    (void)stopped;
    TGV_CUDA(cudaMemcpyAsync(u_dev, c->st.u, n * 4, cudaMemcpyDeviceToDevice, s));
    poisson_integrate(plan, c->st.v[0], c->st.v[1], c->st.three ? c->st.v[2] : nullptr, l_dev,
                      c->prm.dct_mode, c->prm.poisson_eigen, s);
    deshade_epilogue(u_dev, l_dev, mask_dev, n, mask_shading, clamp, add_back, r_dev, s, masked);
    if (log_domain) {
        exp_inplace(u_dev, n, s);
        exp_inplace(l_dev, n, s);
        exp_inplace(r_dev, n, s);
    }
}

// TGVKDeshadeDownsampledProcessor::processTGVKL1Cuda
// (tgvk_deshade_downsampled/TGVKDeshadeDownsampledProcessor.cpp:30-129) and, with
// not_masked, TGVKDeshadeDownsampledNotMaskedProcessor::processTGVKL1Cuda (same file
// layout, :30-129), order 2, on device buffers.  Order 2 is what the reference hands
// to its TGV2 processors with alpha0 = alpha[1] and alpha1 = alpha[0]
// (TGVKDeshadeMaskedProcessor.cpp:98-103, TGVKDeshadeProcessor.cpp:137-147, 242-250).
// Returns whether the callback stopped the loop.
bool downsampled_on_device(const float* f, const float* mask, uint32_t w, uint32_t h, uint32_t d,
                           float factor, float lambda, const float* alpha, uint32_t iterations,
                           uint32_t paint_interval, bool clamp, bool add_back, bool not_masked,
                           tgvdct_iteration_callback cb, void* user, float* u_out, float* l_out,
                           float* r_out, float* divv_out, cudaStream_t s) {
    NvtxRange range("tgvdct downsampled deshade");
    const size_t n = (size_t)w * h * d;
    const bool same = factor == 1.f;  // the reference skips both resizes (:65-66, :105-106)
    const uint32_t W = same ? w : resize_factor_extent(w, factor);
    const uint32_t H = same ? h : resize_factor_extent(h, factor);
    const uint32_t D = same ? d : resize_factor_extent(d, factor);
    const size_t m = (size_t)W * H * D;
    // the masked variant multiplies the input by the mask before resizing (:59-60)
    DevBuf fin((!not_masked && mask) ? n : 0);
    const float* src = f;
    if (!not_masked && mask) {
        multiply_fields(f, mask, fin.p, n, s);
        src = fin.p;
    }
    const size_t scratch_bytes =
        same ? 0
             : std::max(resize_scratch_bytes((int)w, (int)h, (int)d, (int)W, (int)H, (int)D),
                        resize_scratch_bytes((int)W, (int)H, (int)D, (int)w, (int)h, (int)d));
    DevBuf scratch((scratch_bytes + 3) / 4);
    DevBuf ds(same ? 0 : m), dsm((same || !mask) ? 0 : m);
    const float* ds_p = src;
    const float* dsm_p = mask;
    if (!same) {
        resize_bspline3(src, (int)w, (int)h, (int)d, ds.p, (int)W, (int)H, (int)D, scratch.p, s);
        ds_p = ds.p;
        if (mask) {
            resize_bspline3(mask, (int)w, (int)h, (int)d, dsm.p, (int)W, (int)H, (int)D,
                            scratch.p, s);
            dsm_p = dsm.p;
        }
    }
    tgvdct_params q;
    tgvdct_params_init(&q);
    q.width = W;
    q.height = H;
    q.depth = D;
    q.lambda = lambda;
    q.alpha0 = alpha[1];
    q.alpha1 = alpha[0];
    q.iteration_count = iterations;
    q.paint_iteration_interval = paint_interval;
    q.geometry = D == 1 ? TGVDCT_GEOMETRY_2D : TGVDCT_GEOMETRY_3D;
    CtxGuard g;
    create_into(&q, &g.c);
    tgvdct_context* c = g.c;
    DevBuf du(m), dl(m), dr(m);
    if (!not_masked) {
        // the masked processor: a missing mask means every voxel (TGVDeshadeMaskedProcessor.cpp:102-106)
        DevBuf ones(dsm_p ? 0 : m);
        if (!dsm_p) {
            fill_field(ones.p, 1.f, m, s);
            dsm_p = ones.p;
        }
        set_domain(c, dsm_p, s);
        process_on_device(c, ds_p, nullptr, clamp, add_back, false, du.p, dl.p, dr.p, cb, user, s);
        TGV_CUDA(cudaStreamSynchronize(s));  // `ones` is freed on return
    } else {
        process_on_device(c, ds_p, dsm_p, clamp, add_back, false, du.p, dl.p, dr.p, cb, user, s);
    }
    check_tgv_flag(c, s);
    const bool stopped = c->iterations_run < iterations;
    DevBuf ddiv((divv_out && !same) ? m : 0);
    if (divv_out)
        divergence(plan_of(c), c->st.v[0], c->st.v[1], D > 1 ? c->st.v[2] : nullptr,
                   same ? divv_out : ddiv.p, s);
    if (same) {
        TGV_CUDA(cudaMemcpyAsync(u_out, du.p, n * 4, cudaMemcpyDeviceToDevice, s));
        TGV_CUDA(cudaMemcpyAsync(l_out, dl.p, n * 4, cudaMemcpyDeviceToDevice, s));
    } else {
        resize_bspline3(du.p, (int)W, (int)H, (int)D, u_out, (int)w, (int)h, (int)d, scratch.p, s);
        resize_bspline3(dl.p, (int)W, (int)H, (int)D, l_out, (int)w, (int)h, (int)d, scratch.p, s);
        if (divv_out)
            resize_bspline3(ddiv.p, (int)W, (int)H, (int)D, divv_out, (int)w, (int)h, (int)d,
                            scratch.p, s);
    }
    downsampled_tail(f, mask, l_out, r_out, n, not_masked, clamp, add_back, s);
    TGV_CUDA(cudaStreamSynchronize(s));  // the scratch buffers are freed on return
    return stopped;
}

}  // namespace

namespace {
// The convergence test on a context whose st.f holds the input: every `interval`
// iterations l = integrate(v) (times the mask when given) and, from the second check
// on, one (ncc, time-TV) pair of l against the previous l (FP64, on the device).
// Afterwards the TV of each metric series over the checks, all differences but the
// last (TGVDeshadeProcessor.cpp:548-568).
void convergence_on_context(tgvdct_context* c, const float* mask_dev, uint32_t interval,
                            std::vector<double>& ncc, std::vector<double>& tv, double* mt,
                            cudaStream_t s) {
    const size_t n = voxels(c->prm);
    c->prm.paint_iteration_interval = interval;
    const uint32_t checks = interval > 0 ? c->prm.iteration_count / interval + 1 : 0;
    DevBuf lbuf(2 * n), rbuf(n);
    double* dmem = nullptr;
    const size_t ndbl = 8 + 2 * (size_t)checks;
    TGV_CUDA(cudaMalloc(&dmem, ndbl * sizeof(double)));
    struct Free {
        double* p;
        ~Free() { cudaFree(p); }
    } fr{dmem};
    TGV_CUDA(cudaMemsetAsync(dmem, 0, ndbl * sizeof(double), s));
    double* sums = dmem;
    double* hist = dmem + 8;
    DctPlan* plan = plan_of(c);
    float* cur = lbuf.p;
    float* prev = lbuf.p + n;
    bool have_prev = false;
    uint32_t count = 0;
    run_loop(c, s, true, [&](uint32_t) {
        poisson_integrate(plan, c->st.v[0], c->st.v[1], c->st.three ? c->st.v[2] : nullptr, cur,
                          c->prm.dct_mode, c->prm.poisson_eigen, s);
        if (mask_dev)  // l *= mask (TGVDeshadeProcessor.cpp:85-89); r is not used
            deshade_epilogue(c->st.u, cur, mask_dev, n, true, false, false, rbuf.p, s);
        if (have_prev && count < checks) convergence_metrics(cur, prev, n, sums, hist + 2 * count++, s);
        have_prev = true;
        std::swap(cur, prev);
        return false;
    });
    std::vector<double> h(2 * (size_t)count);
    if (count)
        TGV_CUDA(cudaMemcpyAsync(h.data(), hist, h.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
    TGV_CUDA(cudaStreamSynchronize(s));
    ncc.resize(count);
    tv.resize(count);
    for (uint32_t k = 0; k < count; ++k) {
        ncc[k] = h[2 * k];
        tv[k] = h[2 * k + 1];
    }
    for (int m = 0; m < 2; ++m) {
        const std::vector<double>& v = m == 0 ? ncc : tv;
        double acc = 0.0;
        for (size_t i = 0; i + 2 < v.size(); ++i) acc += std::fabs(v[i + 1] - v[i]);
        mt[m] = acc;
    }
}
}  // namespace

namespace {
template <class Body>
tgvdct_status with_plan(uint32_t w, uint32_t h, uint32_t d, Body&& body) {
    return guarded([&] {
        TGV_REQUIRE(w >= 1 && h >= 1 && d >= 1, "width, height, depth must be >= 1");
        check_device();
        DctPlan* plan = dct_plan_create((int)w, (int)h, (int)d);
        struct PlanGuard {
            DctPlan* p;
            ~PlanGuard() { dct_plan_destroy(p); }
        } pg{plan};
        body(plan, (size_t)w * h * d);
        TGV_CUDA(cudaStreamSynchronize(0));
        if (!dct_tc_check(plan, 0)) {
            set_error("a tensor-core DCT pass timed out waiting on its pipeline");
            return TGVDCT_ERR_TIMEOUT;
        }
        return TGVDCT_OK;
    });
}
}  // namespace

extern "C" {

const char* tgvdct_version(void) { return "tgvdct 0.1 (sm_103a)"; }

const char* tgvdct_status_string(tgvdct_status s) {
    switch (s) {
        case TGVDCT_OK: return "ok";
        case TGVDCT_ERR_BAD_ARG: return "bad argument";
        case TGVDCT_ERR_OOM: return "out of memory";
        case TGVDCT_ERR_CUDA: return "CUDA error";
        case TGVDCT_ERR_NO_DEVICE: return "no suitable CUDA device";
        case TGVDCT_ERR_UNSUPPORTED: return "unsupported mode";
        case TGVDCT_STOPPED: return "stopped before the iteration count";
        case TGVDCT_ERR_TIMEOUT: return "a bounded wait in a kernel ran out";
    }
    return "unknown status";
}

const char* tgvdct_last_error(void) { return tgvdct::g_last_error.c_str(); }

void tgvdct_params_init(tgvdct_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    // defaults of the TGV deshade widget (tgv_deshade/TGVDeshadeWidget.ui:43-119)
    p->lambda = 1.f;
    p->alpha0 = 2.f;
    p->alpha1 = 1.f;
    p->iteration_count = 10000;
    const float step = (float)(1.0 / std::sqrt(20.0));  // tgv2_l1_deshade.cu:148-150
    p->tau = step;
    p->sigma = step;
    p->theta = 1.f;
    p->data_term = TGVDCT_DATA_L1;
    p->geometry = TGVDCT_GEOMETRY_3D;
    p->state_precision = TGVDCT_STATE_FP32;
    p->dct_mode = TGVDCT_DCT_FP32;
    p->poisson_eigen = TGVDCT_EIGEN_REFERENCE;
}

size_t tgvdct_workspace_bytes(const tgvdct_params* p) {
    if (!p) return 0;
    return tgv_state_bytes((int)p->width, (int)p->height, (int)p->depth,
                           p->geometry == TGVDCT_GEOMETRY_3D, p->state_precision,
                           kernel_of(*p)) +
           dct_plan_bytes((int)p->width, (int)p->height, (int)p->depth);
}

tgvdct_status tgvdct_create(const tgvdct_params* p, tgvdct_context** out) {
    return guarded([&] {
        create_into(p, out);
        return TGVDCT_OK;
    });
}

tgvdct_status tgvdct_destroy(tgvdct_context* ctx) {
    destroy_ctx(ctx);
    return TGVDCT_OK;
}

tgvdct_status tgvdct_set_params(tgvdct_context* ctx, const tgvdct_params* p) {
    return guarded([&] {
        TGV_REQUIRE(ctx != nullptr, "null context");
        validate(p);
        TGV_REQUIRE(p->width == ctx->prm.width && p->height == ctx->prm.height &&
                        p->depth == ctx->prm.depth,
                    "set_params cannot change the shape");
        TGV_REQUIRE(p->geometry == ctx->prm.geometry &&
                        p->state_precision == ctx->prm.state_precision &&
                        kernel_of(*p) == kernel_of(ctx->prm),
                    "set_params cannot change geometry, state precision or iteration kernel");
        ctx->prm = *p;
        const int zchunk = ctx->st.domain ? masked_zchunk(*p) : auto_zchunk(*p);
        if (zchunk != ctx->st.zchunk) {
            ctx->st.zchunk = zchunk;
            // the per-block domain flags follow the fused kernel's grid
            if (ctx->st.domain) tgv_build_tile_flags(ctx->st, ctx->tile_flags, 0);
        }
        return TGVDCT_OK;
    });
}

uint32_t tgvdct_iterations_run(const tgvdct_context* ctx) { return ctx ? ctx->iterations_run : 0; }

uint64_t tgvdct_loop_launches(const tgvdct_context* ctx) { return ctx ? ctx->loop_launches : 0; }

tgvdct_status tgvdct_tgv2_run_dev(tgvdct_context* c, const float* f_dev, float* u_dev,
                                  float* v_x_dev, float* v_y_dev, float* v_z_dev,
                                  tgvdct_iteration_callback cb, void* user, void* stream) {
    return guarded([&] {
        TGV_REQUIRE(c != nullptr, "null context");
        TGV_REQUIRE(f_dev && u_dev && v_x_dev && v_y_dev, "null device buffer");
        TGV_REQUIRE(v_z_dev || !c->st.three, "v_z is required for 3-D geometry");
        cudaStream_t s = (cudaStream_t)stream;
        const size_t n = voxels(c->prm);
        TGV_CUDA(cudaMemcpyAsync(c->st.f, f_dev, n * 4, cudaMemcpyDeviceToDevice, s));
        const bool stopped = run_loop(c, s, cb != nullptr, [&](uint32_t it) {
            return deliver(c, cb, user, it, c->st.u, c->st.v[0], c->st.v[1],
                           c->st.three ? c->st.v[2] : nullptr, s) != 0;
        });
        TGV_CUDA(cudaMemcpyAsync(u_dev, c->st.u, n * 4, cudaMemcpyDeviceToDevice, s));
        TGV_CUDA(cudaMemcpyAsync(v_x_dev, c->st.v[0], n * 4, cudaMemcpyDeviceToDevice, s));
        TGV_CUDA(cudaMemcpyAsync(v_y_dev, c->st.v[1], n * 4, cudaMemcpyDeviceToDevice, s));
        if (v_z_dev) {
            if (c->st.three)
                TGV_CUDA(cudaMemcpyAsync(v_z_dev, c->st.v[2], n * 4, cudaMemcpyDeviceToDevice, s));
            else
                TGV_CUDA(cudaMemsetAsync(v_z_dev, 0, n * 4, s));
        }
        return stopped ? TGVDCT_STOPPED : TGVDCT_OK;
    });
}

size_t tgvdct_state_bytes(const tgvdct_context* c) {
    return c ? tgv_snapshot_bytes(c->st) : 0;
}

tgvdct_status tgvdct_state_save_dev(tgvdct_context* c, void* dst_dev, void* stream) {
    return guarded([&] {
        TGV_REQUIRE(c != nullptr, "null context");
        TGV_REQUIRE(dst_dev != nullptr, "null device buffer");
        tgv_snapshot_save(c->st, dst_dev, (cudaStream_t)stream);
        return TGVDCT_OK;
    });
}

tgvdct_status tgvdct_state_load_dev(tgvdct_context* c, const void* src_dev, void* stream) {
    return guarded([&] {
        TGV_REQUIRE(c != nullptr, "null context");
        TGV_REQUIRE(src_dev != nullptr, "null device buffer");
        tgv_snapshot_load(c->st, src_dev, (cudaStream_t)stream);
        return TGVDCT_OK;
    });
}

tgvdct_status tgvdct_tgv2_resume_dev(tgvdct_context* c, float* u_dev, float* v_x_dev,
                                     float* v_y_dev, float* v_z_dev,
                                     tgvdct_iteration_callback cb, void* user, void* stream) {
    return guarded([&] {
        TGV_REQUIRE(c != nullptr, "null context");
        TGV_REQUIRE(u_dev && v_x_dev && v_y_dev, "null device buffer");
        TGV_REQUIRE(v_z_dev || !c->st.three, "v_z is required for 3-D geometry");
        cudaStream_t s = (cudaStream_t)stream;
        const size_t n = voxels(c->prm);
        const bool stopped = run_loop(
            c, s, cb != nullptr,
            [&](uint32_t it) {
                return deliver(c, cb, user, it, c->st.u, c->st.v[0], c->st.v[1],
                               c->st.three ? c->st.v[2] : nullptr, s) != 0;
            },
            false);
        TGV_CUDA(cudaMemcpyAsync(u_dev, c->st.u, n * 4, cudaMemcpyDeviceToDevice, s));
        TGV_CUDA(cudaMemcpyAsync(v_x_dev, c->st.v[0], n * 4, cudaMemcpyDeviceToDevice, s));
        TGV_CUDA(cudaMemcpyAsync(v_y_dev, c->st.v[1], n * 4, cudaMemcpyDeviceToDevice, s));
        if (v_z_dev) {
            if (c->st.three)
                TGV_CUDA(cudaMemcpyAsync(v_z_dev, c->st.v[2], n * 4, cudaMemcpyDeviceToDevice, s));
            else
                TGV_CUDA(cudaMemsetAsync(v_z_dev, 0, n * 4, s));
        }
        return stopped ? TGVDCT_STOPPED : TGVDCT_OK;
    });
}

// ---- z-slab decomposition: state access by planes, single steps, Poisson pieces ----
}  // extern "C"
namespace {

// The state field a field-mask bit names (current stencil set for ubar, vbar, p, q),
// with its element size; null when the state has no such field (v_z in 2-D).
void* state_field(const TgvState& s, int bit, size_t* elem) {
    const TgvStencilFields& F = s.now();
    *elem = 4;
    switch (bit) {
        case 0: return s.f;
        case 1: return s.u;
        case 2: case 3: case 4: return s.v[bit - 2];
        case 5: return F.ubar;
        case 6: case 7: case 8: return F.vbar[bit - 6];
        default: break;
    }
    *elem = s.precision == TGVDCT_STATE_FP32 ? 4 : 2;
    if (bit >= 9 && bit <= 11) return F.p[bit - 9];
    if (bit >= 12 && bit <= 17) return F.q[bit - 12];
    return nullptr;
}

// Runs fn(field pointer, bytes of one plane) over the fields of `mask` in bit order.
template <class Fn>
void for_each_masked_field(const TgvState& s, uint32_t mask, Fn&& fn) {
    TGV_REQUIRE((mask & ~TGVDCT_FIELD_ALL) == 0, "unknown bits in the field mask");
    const size_t plane = (size_t)s.W * s.H;
    for (int bit = 0; bit < 18; ++bit) {
        if (!(mask & (1u << bit))) continue;
        size_t e = 0;
        void* f = state_field(s, bit, &e);
        TGV_REQUIRE(f != nullptr, "the field mask names a field this state does not have");
        fn((char*)f, plane * e);
    }
}

}  // namespace
extern "C" {

tgvdct_status tgvdct_state_init_dev(tgvdct_context* c, const float* f_dev, void* stream) {
    return guarded([&] {
        TGV_REQUIRE(c != nullptr, "null context");
        TGV_REQUIRE(f_dev != nullptr, "null device buffer");
        cudaStream_t s = (cudaStream_t)stream;
        TGV_CUDA(cudaMemcpyAsync(c->st.f, f_dev, voxels(c->prm) * 4, cudaMemcpyDeviceToDevice, s));
        tgv_state_init(c->st, s);
        c->iterations_run = 0;
        return TGVDCT_OK;
    });
}

tgvdct_status tgvdct_tgv2_step_dev(tgvdct_context* c, uint32_t iterations, void* stream) {
    return guarded([&] {
        TGV_REQUIRE(c != nullptr, "null context");
        const TgvStep k = step_of(c->prm);
        c->loop_launches = (uint64_t)tgv_iterate_n(c->st, k, iterations, (cudaStream_t)stream);
        c->iterations_run = iterations;
        return TGVDCT_OK;
    });
}

size_t tgvdct_state_planes_bytes(const tgvdct_context* c, uint32_t field_mask,
                                 uint32_t plane_count) {
    if (!c) return 0;
    size_t b = 0;
    try {
        for_each_masked_field(c->st, field_mask,
                              [&](char*, size_t plane_bytes) { b += plane_bytes * plane_count; });
    } catch (const Error&) {
        return 0;
    }
    return b;
}

tgvdct_status tgvdct_state_read_dev(tgvdct_context* c, uint32_t field_mask, uint32_t plane_begin,
                                    uint32_t plane_count, void* dst_dev, void* stream) {
    return guarded([&] {
        TGV_REQUIRE(c != nullptr, "null context");
        TGV_REQUIRE(dst_dev != nullptr, "null device buffer");
        TGV_REQUIRE((uint64_t)plane_begin + plane_count <= c->prm.depth, "planes out of range");
        char* d = (char*)dst_dev;
        for_each_masked_field(c->st, field_mask, [&](char* f, size_t plane_bytes) {
            const size_t n = plane_bytes * plane_count;
            TGV_CUDA(cudaMemcpyAsync(d, f + plane_bytes * plane_begin, n,
                                     cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
            d += n;
        });
        return TGVDCT_OK;
    });
}

tgvdct_status tgvdct_state_write_dev(tgvdct_context* c, uint32_t field_mask,
                                     uint32_t plane_begin, uint32_t plane_count,
                                     const void* src_dev, void* stream) {
    return guarded([&] {
        TGV_REQUIRE(c != nullptr, "null context");
        TGV_REQUIRE(src_dev != nullptr, "null device buffer");
        TGV_REQUIRE((uint64_t)plane_begin + plane_count <= c->prm.depth, "planes out of range");
        const char* d = (const char*)src_dev;
        for_each_masked_field(c->st, field_mask, [&](char* f, size_t plane_bytes) {
            const size_t n = plane_bytes * plane_count;
            TGV_CUDA(cudaMemcpyAsync(f + plane_bytes * plane_begin, d, n,
                                     cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
            d += n;
        });
        return TGVDCT_OK;
    });
}

tgvdct_status tgvdct_slab_poisson_xy_dev(tgvdct_context* c, const float* v_x_dev,
                                         const float* v_y_dev, const float* v_z_dev,
                                         float* out_dev, void* stream) {
    return guarded([&] {
        TGV_REQUIRE(c != nullptr, "null context");
        TGV_REQUIRE(v_x_dev && v_y_dev && v_z_dev && out_dev, "null device buffer");
        TGV_REQUIRE(c->prm.depth > 1 && c->st.three, "a slab is a 3-D volume of depth > 1");
        if (c->prm.dct_mode != TGVDCT_DCT_FP32) {
            set_error("the slab Poisson passes run the FP32 contractions only");
            return TGVDCT_ERR_UNSUPPORTED;
        }
        slab_poisson_xy(plan_of(c), v_x_dev, v_y_dev, v_z_dev, out_dev, (cudaStream_t)stream);
        return TGVDCT_OK;
    });
}

tgvdct_status tgvdct_slab_poisson_inverse_yx_dev(tgvdct_context* c, const float* in_dev,
                                                 float* out_dev, uint32_t plane_count,
                                                 uint32_t total_depth, void* stream) {
    return guarded([&] {
        TGV_REQUIRE(c != nullptr, "null context");
        TGV_REQUIRE(in_dev && out_dev, "null device buffer");
        TGV_REQUIRE(plane_count >= 1 && plane_count <= c->prm.depth, "plane_count out of range");
        TGV_REQUIRE(total_depth >= plane_count, "total_depth below plane_count");
        if (c->prm.dct_mode != TGVDCT_DCT_FP32) {
            set_error("the slab Poisson passes run the FP32 contractions only");
            return TGVDCT_ERR_UNSUPPORTED;
        }
        // the single-volume scale 1 / (8 W H D) of the whole volume
        const float scale =
            (float)(1.0 / ((double)c->prm.width * c->prm.height * total_depth * 8.0));
        slab_poisson_inverse_yx(plan_of(c), in_dev, out_dev, (int)plane_count, scale,
                                (cudaStream_t)stream);
        return TGVDCT_OK;
    });
}

struct tgvdct_pencil {
    DctPlan* plan = nullptr;
    uint64_t columns = 0;
};

tgvdct_status tgvdct_pencil_create(uint32_t width, uint32_t height, uint32_t depth,
                                   uint64_t columns, tgvdct_pencil** out) {
    return guarded([&] {
        TGV_REQUIRE(out != nullptr, "null output pointer");
        *out = nullptr;
        TGV_REQUIRE(width >= 1 && height >= 1 && depth >= 2, "a pencil needs depth >= 2");
        TGV_REQUIRE(columns >= 1 && columns <= (uint64_t)width * height,
                    "columns must be in 1 .. width * height");
        TGV_REQUIRE((uint64_t)depth * columns < ((uint64_t)1 << 31), "pencil too large");
        auto* p = new tgvdct_pencil();
        try {
            p->plan = dct_plan_create((int)width, (int)height, (int)depth,
                                      (size_t)depth * columns);
        } catch (...) {
            delete p;
            throw;
        }
        p->columns = columns;
        *out = p;
        return TGVDCT_OK;
    });
}

tgvdct_status tgvdct_pencil_destroy(tgvdct_pencil* p) {
    if (!p) return TGVDCT_OK;
    dct_plan_destroy(p->plan);
    delete p;
    return TGVDCT_OK;
}

tgvdct_status tgvdct_pencil_poisson_z_dev(tgvdct_pencil* p, const float* in_dev, float* out_dev,
                                          uint64_t column_begin, int32_t poisson_eigen,
                                          void* stream) {
    return guarded([&] {
        TGV_REQUIRE(p != nullptr, "null pencil");
        TGV_REQUIRE(in_dev && out_dev, "null device buffer");
        TGV_REQUIRE(column_begin + p->columns <= (uint64_t)p->plan->W * p->plan->H,
                    "the pencil's columns run past the plane");
        TGV_REQUIRE(poisson_eigen == TGVDCT_EIGEN_REFERENCE ||
                        poisson_eigen == TGVDCT_EIGEN_ACCURATE,
                    "unknown Poisson eigenvalue mode");
        pencil_poisson_z(p->plan, in_dev, out_dev, (long long)p->columns, (long long)column_begin,
                         poisson_eigen, (cudaStream_t)stream);
        return TGVDCT_OK;
    });
}

tgvdct_status tgvdct_tgv2_forward_checkpointed_dev(tgvdct_context* c, const float* f_dev,
                                                   float* u_dev, float* v_x_dev,
                                                   float* v_y_dev, float* v_z_dev,
                                                   uint32_t checkpoint_every, void* stream) {
    return guarded([&] {
        TGV_REQUIRE(c != nullptr, "null context");
        TGV_REQUIRE(f_dev && u_dev && v_x_dev && v_y_dev && v_z_dev, "null device buffer");
        TGV_REQUIRE(checkpoint_every >= 1, "checkpoint_every must be >= 1");
        require_reverse_mode(c);
        cudaStream_t s = (cudaStream_t)stream;
        const size_t n = voxels(c->prm);
        const uint32_t K = c->prm.iteration_count;
        const uint32_t count = (K + checkpoint_every - 1) / checkpoint_every;
        c->have_ckpt = false;
        // the states at iterations 0, k, 2k, ... and the final state (index count)
        if (ensure_block(&c->ckpt_block, &c->ckpt_bytes,
                         (size_t)(count + 1) * tgv_full_state_bytes(n)))
            c->step_cache.reset();
        TGV_CUDA(cudaMemcpyAsync(c->st.f, f_dev, n * 4, cudaMemcpyDeviceToDevice, s));
        tgv_state_init(c->st, s);
        const TgvStep k = step_of(c->prm);
        for (uint32_t it = 0; it < K;) {
            // the iterations between two checkpoints as one stretch
            tgv_save_state(c->st, full_state_at(c->ckpt_block, it / checkpoint_every, n), s);
            const uint32_t len = std::min(checkpoint_every, K - it);
            tgv_iterate_n(c->st, k, len, s);
            it += len;
        }
        tgv_save_state(c->st, full_state_at(c->ckpt_block, count, n), s);
        c->iterations_run = K;
        TGV_CUDA(cudaMemcpyAsync(u_dev, c->st.u, n * 4, cudaMemcpyDeviceToDevice, s));
        float* vo[3] = {v_x_dev, v_y_dev, v_z_dev};
        for (int a = 0; a < 3; ++a)
            TGV_CUDA(cudaMemcpyAsync(vo[a], c->st.v[a], n * 4, cudaMemcpyDeviceToDevice, s));
        c->ckpt_every = checkpoint_every;
        c->ckpt_K = K;
        c->ckpt_count = count;
        c->have_ckpt = true;
        return TGVDCT_OK;
    });
}

namespace {
// The reverse sweep's passes for the context's iteration kernel: the fused adjoint pass
// (R3 of one iteration with R1 and R2 of the one before) for shifted passes, and for
// the automatic choice when its grid fills the GPU; separate passes otherwise.
AdjointPasses adjoint_passes(const tgvdct_params& p) {
    switch (p.iteration_kernel) {
        case TGVDCT_KERNEL_FUSED_SHIFTED: return ADJ_FUSED;
        case TGVDCT_KERNEL_AUTO: return ADJ_FUSED_LARGE;
        default: return ADJ_SEPARATE;
    }
}

// The reverse sweep over every segment, last to first, then the u_0 = ubar_0 = f term.
// The fused adjoint passes alternate between the adjoint states A and A2 (each segment
// swaps the descriptors as it goes); the sweep's result is in whichever one the last
// segment left current, which is the same one on every replay of a captured sweep.
void backward_segments(tgvdct_context* c, const TgvStep& k, const TgvFullDev& A0,
                       const TgvFullDev& A20, float* uta, float* const* va, float* grad_f,
                       double* gp, cudaStream_t s) {
    NvtxRange range("tgvdct reverse sweep");
    const size_t n = voxels(c->prm);
    const uint32_t every = c->ckpt_every, K = c->ckpt_K;
    TgvFullDev A = A0, A2 = A20;
    std::vector<TgvFullDev> states(every + 1);
    for (int seg = (int)c->ckpt_count - 1; seg >= 0; --seg) {
        const uint32_t k0 = (uint32_t)seg * every, k1 = k0 + every < K ? k0 + every : K;
        const int len = (int)(k1 - k0);
        states[0] = full_state_at(c->ckpt_block, seg, n);
        for (int j = 1; j < len; ++j) states[j] = full_state_at(c->seg_block, j - 1, n);
        states[len] = full_state_at(c->ckpt_block, seg + 1, n);
        for (int j = 0; j + 1 < len; ++j)
            tgv_step_fp32(c->st, k, states[j], states[j + 1], c->step_cache, s);
        tgv_adjoint_segment(c->st, k, states.data(), len, adjoint_passes(c->prm), A, A2, uta,
                            va, grad_f, gp, s);
    }
    tgv_adjoint_finish(grad_f, A, n, s);
}

// The backward sweep as a CUDA graph (a few hundred launches of tens of microseconds
// each at small volumes), captured on first use and replayed while the buffers, the
// segmentation, the step and the z-chunk stay the same.  Null when capture fails; the
// caller then runs the sweep directly.  The iteration kernel's shared-memory
// attribute was set by the checkpointed forward that every backward follows.
cudaGraphExec_t backward_graph(tgvdct_context* c, const TgvStep& k, const TgvFullDev& A,
                               const TgvFullDev& A2, float* uta, float* const* va,
                               float* grad_f, double* gp) {
    tgvdct_context::BwdKey key;
    key.ckpt = c->ckpt_block;
    key.seg = c->seg_block;
    key.adj = c->adj_block;
    key.every = c->ckpt_every;
    key.K = c->ckpt_K;
    key.count = c->ckpt_count;
    key.zchunk = c->st.zchunk;
    key.step = k;
    key.passes = adjoint_passes(c->prm);
    const auto& o = c->bwd_key;
    if (c->bwd_graph && o.ckpt == key.ckpt && o.seg == key.seg && o.adj == key.adj &&
        o.every == key.every && o.K == key.K && o.count == key.count && o.zchunk == key.zchunk &&
        o.passes == key.passes && same_step(o.step, k))
        return c->bwd_graph;
    if (c->bwd_graph) {
        cudaGraphExecDestroy(c->bwd_graph);
        c->bwd_graph = nullptr;
    }
    if (!c->capture_stream &&
        cudaStreamCreateWithFlags(&c->capture_stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (cudaStreamBeginCapture(c->capture_stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    cudaGraph_t g = nullptr;
    bool built = true;
    try {
        backward_segments(c, k, A, A2, uta, va, grad_f, gp, c->capture_stream);
    } catch (...) {
        built = false;
    }
    const cudaError_t e = cudaStreamEndCapture(c->capture_stream, &g);
    if (!built || e != cudaSuccess || !g) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        return nullptr;
    }
    const cudaError_t ie = cudaGraphInstantiate(&c->bwd_graph, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) {
        cudaGetLastError();
        c->bwd_graph = nullptr;
        return nullptr;
    }
    c->bwd_key = key;
    return c->bwd_graph;
}
}  // namespace

tgvdct_status tgvdct_tgv2_backward_dev(tgvdct_context* c, const float* grad_u_dev,
                                       const float* grad_v_x_dev, const float* grad_v_y_dev,
                                       const float* grad_v_z_dev, float* grad_f_dev,
                                       double* grad_params_dev, void* stream) {
    return guarded([&] {
        TGV_REQUIRE(c != nullptr, "null context");
        TGV_REQUIRE(grad_f_dev && grad_params_dev, "null device buffer");
        TGV_REQUIRE(c->have_ckpt, "no checkpointed forward run on this context");
        require_reverse_mode(c);
        cudaStream_t s = (cudaStream_t)stream;
        const size_t n = voxels(c->prm);
        const uint32_t every = c->ckpt_every;
        // a segment [k0, k1) reads S_k0 and S_k1 from the checkpoints and recomputes
        // the k1 - k0 - 1 states between them
        if (every > 1 &&
            ensure_block(&c->seg_block, &c->seg_bytes, (size_t)(every - 1) * tgv_full_state_bytes(n)))
            c->step_cache.reset();
        // two adjoint states (the fused passes write from one into the other), scratch
        // a(u~) and a(v'), and the sweep's own d/df and d/d(lambda, alpha0, alpha1)
        // (copied to the caller's buffers at the end, so a captured sweep does not depend
        // on them)
        const size_t field = (n * 4 + 255) & ~size_t(255);
        ensure_block(&c->adj_block, &c->adj_bytes, 2 * tgv_full_state_bytes(n) + 5 * field + 256);
        TgvFullDev A = full_state_at(c->adj_block, 0, n);
        TgvFullDev A2 = full_state_at(c->adj_block, 1, n);
        char* scratch = (char*)c->adj_block + 2 * tgv_full_state_bytes(n);
        float* uta = (float*)scratch;
        float* va[3] = {(float*)(scratch + field), (float*)(scratch + 2 * field),
                        (float*)(scratch + 3 * field)};
        float* gf = (float*)(scratch + 4 * field);
        double* gp = (double*)(scratch + 5 * field);
        tgv_full_state_zero(A, n, s);
        if (grad_u_dev) TGV_CUDA(cudaMemcpyAsync(A.u, grad_u_dev, n * 4, cudaMemcpyDeviceToDevice, s));
        const float* gv[3] = {grad_v_x_dev, grad_v_y_dev, grad_v_z_dev};
        for (int a = 0; a < 3; ++a)
            if (gv[a]) TGV_CUDA(cudaMemcpyAsync(A.v[a], gv[a], n * 4, cudaMemcpyDeviceToDevice, s));
        TGV_CUDA(cudaMemsetAsync(gf, 0, n * 4, s));
        TGV_CUDA(cudaMemsetAsync(gp, 0, 3 * sizeof(double), s));
        const TgvStep k = step_of(c->prm);
        if (cudaGraphExec_t g = backward_graph(c, k, A, A2, uta, va, gf, gp))
            TGV_CUDA(cudaGraphLaunch(g, s));
        else
            backward_segments(c, k, A, A2, uta, va, gf, gp, s);
        TGV_CUDA(cudaMemcpyAsync(grad_f_dev, gf, n * 4, cudaMemcpyDeviceToDevice, s));
        TGV_CUDA(cudaMemcpyAsync(grad_params_dev, gp, 3 * sizeof(double), cudaMemcpyDeviceToDevice,
                                 s));
        return TGVDCT_OK;
    });
}

tgvdct_status tgvdct_tgv2_l1_deshade_launch(const float* f_host, uint32_t width, uint32_t height,
                                            uint32_t depth, float lambda,
                                            uint32_t iteration_count,
                                            uint32_t paint_iteration_interval,
                                            int cuda_block_dimension,
                                            tgvdct_iteration_callback callback, void* user,
                                            float alpha0, float alpha1, float* u_host,
                                            float* v_x_host, float* v_y_host, float* v_z_host) {
    (void)cuda_block_dimension;
    return guarded([&] {
        TGV_REQUIRE(f_host && u_host && v_x_host && v_y_host && v_z_host, "null host buffer");
        tgvdct_params p;
        tgvdct_params_init(&p);
        p.width = width;
        p.height = height;
        p.depth = depth;
        p.lambda = lambda;
        p.alpha0 = alpha0;
        p.alpha1 = alpha1;
        p.iteration_count = iteration_count;
        p.paint_iteration_interval = paint_iteration_interval;
        validate(&p);
        HostLease g(p, HK_DESHADE_LAUNCH, 0);
        tgvdct_context* c = g.c;
        const size_t n = voxels(p);
        cudaStream_t s = 0;
        TGV_CUDA(cudaMemcpyAsync(c->st.f, f_host, n * 4, cudaMemcpyHostToDevice, s));
        const bool stopped = run_loop(c, s, callback != nullptr, [&](uint32_t it) {
            return deliver(c, callback, user, it, c->st.u, c->st.v[0], c->st.v[1], c->st.v[2], s) != 0;
        });
        TGV_CUDA(cudaMemcpyAsync(u_host, c->st.u, n * 4, cudaMemcpyDeviceToHost, s));
        TGV_CUDA(cudaMemcpyAsync(v_x_host, c->st.v[0], n * 4, cudaMemcpyDeviceToHost, s));
        TGV_CUDA(cudaMemcpyAsync(v_y_host, c->st.v[1], n * 4, cudaMemcpyDeviceToHost, s));
        TGV_CUDA(cudaMemcpyAsync(v_z_host, c->st.v[2], n * 4, cudaMemcpyDeviceToHost, s));
        check_tgv_flag(c, s);
        g.commit();
        return stopped ? TGVDCT_STOPPED : TGVDCT_OK;
    });
}

tgvdct_status tgvdct_tgv2_l1_deshade_launch_2d(const float* f_host, uint32_t width,
                                               uint32_t height, float lambda,
                                               uint32_t iteration_count,
                                               uint32_t paint_iteration_interval,
                                               tgvdct_iteration_callback callback, void* user,
                                               float alpha0, float alpha1, float* u_host,
                                               float* v_x_host, float* v_y_host) {
    return guarded([&] {
        TGV_REQUIRE(f_host && u_host && v_x_host && v_y_host, "null host buffer");
        tgvdct_params p;
        tgvdct_params_init(&p);
        p.width = width;
        p.height = height;
        p.depth = 1;
        p.geometry = TGVDCT_GEOMETRY_2D;
        p.lambda = lambda;
        p.alpha0 = alpha0;
        p.alpha1 = alpha1;
        p.iteration_count = iteration_count;
        p.paint_iteration_interval = paint_iteration_interval;
        validate(&p);
        HostLease g(p, HK_DESHADE_LAUNCH, 0);
        tgvdct_context* c = g.c;
        const size_t n = voxels(p);
        cudaStream_t s = 0;
        TGV_CUDA(cudaMemcpyAsync(c->st.f, f_host, n * 4, cudaMemcpyHostToDevice, s));
        const bool stopped = run_loop(c, s, callback != nullptr, [&](uint32_t it) {
            return deliver(c, callback, user, it, c->st.u, c->st.v[0], c->st.v[1], nullptr, s) != 0;
        });
        TGV_CUDA(cudaMemcpyAsync(u_host, c->st.u, n * 4, cudaMemcpyDeviceToHost, s));
        TGV_CUDA(cudaMemcpyAsync(v_x_host, c->st.v[0], n * 4, cudaMemcpyDeviceToHost, s));
        TGV_CUDA(cudaMemcpyAsync(v_y_host, c->st.v[1], n * 4, cudaMemcpyDeviceToHost, s));
        check_tgv_flag(c, s);
        g.commit();
        return stopped ? TGVDCT_STOPPED : TGVDCT_OK;
    });
}

tgvdct_status tgvdct_tgv2_run(const tgvdct_params* p, const float* f_host, float* u_host,
                             float* v_x_host, float* v_y_host, float* v_z_host,
                             tgvdct_iteration_callback callback, void* user) {
    return guarded([&] {
        TGV_REQUIRE(p && f_host && u_host, "null host buffer");
        validate(p);
        HostLease g(*p, HK_RUN, 0);
        tgvdct_context* c = g.c;
        const size_t n = voxels(*p);
        cudaStream_t s = 0;
        TGV_CUDA(cudaMemcpyAsync(c->st.f, f_host, n * 4, cudaMemcpyHostToDevice, s));
        const bool stopped = run_loop(c, s, callback != nullptr, [&](uint32_t it) {
            return deliver(c, callback, user, it, c->st.u, c->st.v[0], c->st.v[1],
                           c->st.three ? c->st.v[2] : nullptr, s) != 0;
        });
        TGV_CUDA(cudaMemcpyAsync(u_host, c->st.u, n * 4, cudaMemcpyDeviceToHost, s));
        float* vh[3] = {v_x_host, v_y_host, v_z_host};
        for (int k = 0; k < 3; ++k) {
            if (!vh[k]) continue;
            if (k == 2 && !c->st.three) std::memset(vh[k], 0, n * 4);
            else TGV_CUDA(cudaMemcpyAsync(vh[k], c->st.v[k], n * 4, cudaMemcpyDeviceToHost, s));
        }
        check_tgv_flag(c, s);
        g.commit();
        return stopped ? TGVDCT_STOPPED : TGVDCT_OK;
    });
}

tgvdct_status tgvdct_tgv2_denoise_launch(const float* f_host, uint32_t width, uint32_t height,
                                         uint32_t depth, int32_t data_term, float lambda,
                                         uint32_t iteration_count, float alpha0, float alpha1,
                                         float* u_host) {
    return guarded([&] {
        TGV_REQUIRE(f_host && u_host, "null host buffer");
        tgvdct_params p;
        tgvdct_params_init(&p);
        p.width = width;
        p.height = height;
        p.depth = depth;
        p.data_term = data_term;
        p.lambda = lambda;
        p.alpha0 = alpha0;
        p.alpha1 = alpha1;
        p.iteration_count = iteration_count;
        validate(&p);
        HostLease g(p, HK_DENOISE_LAUNCH, 0);
        tgvdct_context* c = g.c;
        const size_t n = voxels(p);
        cudaStream_t s = 0;
        TGV_CUDA(cudaMemcpyAsync(c->st.f, f_host, n * 4, cudaMemcpyHostToDevice, s));
        run_loop(c, s, false, [](uint32_t) { return false; });
        TGV_CUDA(cudaMemcpyAsync(u_host, c->st.u, n * 4, cudaMemcpyDeviceToHost, s));
        check_tgv_flag(c, s);
        g.commit();
        return TGVDCT_OK;
    });
}

// ---- Poisson integration and image operations (host buffers) ----------------------


tgvdct_status tgvdct_divergence_launch(const float* dx, const float* dy, const float* dz,
                                       uint32_t width, uint32_t height, uint32_t depth,
                                       float* out) {
    return with_plan(width, height, depth, [&](DctPlan* plan, size_t n) {
        TGV_REQUIRE(dx && dy && out && (dz || depth == 1), "null host buffer");
        DevBuf a(n), b(n), c(depth > 1 ? n : 0), o(n);
        TGV_CUDA(cudaMemcpy(a.p, dx, n * 4, cudaMemcpyHostToDevice));
        TGV_CUDA(cudaMemcpy(b.p, dy, n * 4, cudaMemcpyHostToDevice));
        if (depth > 1) TGV_CUDA(cudaMemcpy(c.p, dz, n * 4, cudaMemcpyHostToDevice));
        divergence(plan, a.p, b.p, c.p, o.p, 0);
        TGV_CUDA(cudaMemcpy(out, o.p, n * 4, cudaMemcpyDeviceToHost));
    });
}

tgvdct_status tgvdct_device_alloc(size_t bytes, void** out) {
    return guarded([&] {
        TGV_REQUIRE(out, "null output pointer");
        *out = nullptr;
        check_device();
        const cudaError_t e = cudaMalloc(out, bytes ? bytes : 1);
        if (e != cudaSuccess) {
            cudaGetLastError();
            set_error(std::string("cudaMalloc: ") + cudaGetErrorString(e));
            return TGVDCT_ERR_OOM;
        }
        return TGVDCT_OK;
    });
}

tgvdct_status tgvdct_device_free(void* p) {
    return guarded([&] {
        if (p) TGV_CUDA(cudaFree(p));
        return TGVDCT_OK;
    });
}

tgvdct_status tgvdct_host_to_device(void* dst_dev, const void* src_host, size_t bytes) {
    return guarded([&] {
        TGV_REQUIRE(dst_dev && src_host, "null buffer");
        TGV_CUDA(cudaMemcpy(dst_dev, src_host, bytes, cudaMemcpyHostToDevice));
        return TGVDCT_OK;
    });
}

tgvdct_status tgvdct_device_to_host(void* dst_host, const void* src_dev, size_t bytes) {
    return guarded([&] {
        TGV_REQUIRE(dst_host && src_dev, "null buffer");
        TGV_CUDA(cudaMemcpy(dst_host, src_dev, bytes, cudaMemcpyDeviceToHost));
        return TGVDCT_OK;
    });
}

tgvdct_status tgvdct_divergence_dev(const float* dx_dev, const float* dy_dev,
                                    const float* dz_dev, uint32_t width, uint32_t height,
                                    uint32_t depth, float* out_dev, void* stream) {
    return guarded([&] {
        TGV_REQUIRE(width >= 1 && height >= 1 && depth >= 1, "width, height, depth must be >= 1");
        TGV_REQUIRE(dx_dev && dy_dev && out_dev && (dz_dev || depth == 1), "null device buffer");
        check_device();
        DctPlan* plan = dct_plan_create((int)width, (int)height, (int)depth);
        struct PlanGuard {
            DctPlan* p;
            ~PlanGuard() { dct_plan_destroy(p); }
        } pg{plan};
        divergence(plan, dx_dev, dy_dev, depth > 1 ? dz_dev : nullptr, out_dev,
                   (cudaStream_t)stream);
        TGV_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
        return TGVDCT_OK;
    });
}

tgvdct_status tgvdct_cosine_transform_launch(const float* in, uint32_t width, uint32_t height,
                                             uint32_t depth, int32_t dct_mode, float* out) {
    return with_plan(width, height, depth, [&](DctPlan* plan, size_t n) {
        TGV_REQUIRE(in && out, "null host buffer");
        DevBuf a(n), o(n);
        TGV_CUDA(cudaMemcpy(a.p, in, n * 4, cudaMemcpyHostToDevice));
        cosine_transform(plan, a.p, o.p, dct_mode, 0);
        TGV_CUDA(cudaMemcpy(out, o.p, n * 4, cudaMemcpyDeviceToHost));
    });
}

tgvdct_status tgvdct_inverse_cosine_transform_launch(const float* in, uint32_t width,
                                                     uint32_t height, uint32_t depth,
                                                     int32_t dct_mode, float* out) {
    return with_plan(width, height, depth, [&](DctPlan* plan, size_t n) {
        TGV_REQUIRE(in && out, "null host buffer");
        DevBuf a(n), o(n);
        TGV_CUDA(cudaMemcpy(a.p, in, n * 4, cudaMemcpyHostToDevice));
        inverse_cosine_transform(plan, a.p, o.p, dct_mode, 0);
        TGV_CUDA(cudaMemcpy(out, o.p, n * 4, cudaMemcpyDeviceToHost));
    });
}

tgvdct_status tgvdct_solve_poisson_in_cosine_domain_launch(const float* in, uint32_t width,
                                                           uint32_t height, uint32_t depth,
                                                           int32_t poisson_eigen, float* out) {
    return with_plan(width, height, depth, [&](DctPlan* plan, size_t n) {
        TGV_REQUIRE(in && out, "null host buffer");
        DevBuf a(n), o(n);
        TGV_CUDA(cudaMemcpy(a.p, in, n * 4, cudaMemcpyHostToDevice));
        solve_poisson(plan, a.p, o.p, poisson_eigen, 0);
        TGV_CUDA(cudaMemcpy(out, o.p, n * 4, cudaMemcpyDeviceToHost));
    });
}

tgvdct_status tgvdct_integrate_image_gradients_poisson_cosine_transform(
    const float* v_x, const float* v_y, const float* v_z, uint32_t width, uint32_t height,
    uint32_t depth, int32_t dct_mode, int32_t poisson_eigen, float* l_out) {
    return with_plan(width, height, depth, [&](DctPlan* plan, size_t n) {
        TGV_REQUIRE(v_x && v_y && l_out && (v_z || depth == 1), "null host buffer");
        DevBuf a(n), b(n), c(depth > 1 ? n : 0), o(n);
        TGV_CUDA(cudaMemcpy(a.p, v_x, n * 4, cudaMemcpyHostToDevice));
        TGV_CUDA(cudaMemcpy(b.p, v_y, n * 4, cudaMemcpyHostToDevice));
        if (depth > 1) TGV_CUDA(cudaMemcpy(c.p, v_z, n * 4, cudaMemcpyHostToDevice));
        poisson_integrate(plan, a.p, b.p, c.p, o.p, dct_mode, poisson_eigen, 0);
        TGV_CUDA(cudaMemcpy(l_out, o.p, n * 4, cudaMemcpyDeviceToHost));
    });
}

tgvdct_status tgvdct_poisson_integrate_dev(tgvdct_context* c, const float* v_x_dev,
                                           const float* v_y_dev, const float* v_z_dev,
                                           float* l_dev, void* stream) {
    return guarded([&] {
        TGV_REQUIRE(c != nullptr, "null context");
        TGV_REQUIRE(v_x_dev && v_y_dev && l_dev && (v_z_dev || c->prm.depth == 1),
                    "null device buffer");
        poisson_integrate(plan_of(c), v_x_dev, v_y_dev, v_z_dev, l_dev, c->prm.dct_mode,
                          c->prm.poisson_eigen, (cudaStream_t)stream);
        return TGVDCT_OK;
    });
}

tgvdct_status tgvdct_poisson_solve_dev(tgvdct_context* c, const float* rhs_dev, float* l_dev,
                                       void* stream) {
    return guarded([&] {
        TGV_REQUIRE(c != nullptr, "null context");
        TGV_REQUIRE(rhs_dev && l_dev, "null device buffer");
        poisson_solve(plan_of(c), rhs_dev, l_dev, c->prm.dct_mode, c->prm.poisson_eigen,
                      (cudaStream_t)stream);
        return TGVDCT_OK;
    });
}

tgvdct_status tgvdct_poisson_integrate_adjoint_dev(tgvdct_context* c, const float* grad_l_dev,
                                                   float* grad_v_x_dev, float* grad_v_y_dev,
                                                   float* grad_v_z_dev, void* stream) {
    return guarded([&] {
        TGV_REQUIRE(c != nullptr, "null context");
        TGV_REQUIRE(grad_l_dev && grad_v_x_dev && grad_v_y_dev &&
                        (grad_v_z_dev || c->prm.depth == 1),
                    "null device buffer");
        const size_t n = voxels(c->prm);
        DevBuf scratch(n);
        cudaStream_t s = (cudaStream_t)stream;
        poisson_integrate_adjoint(plan_of(c), grad_l_dev, scratch.p, grad_v_x_dev, grad_v_y_dev,
                                  grad_v_z_dev, c->prm.dct_mode, c->prm.poisson_eigen, s);
        if (grad_v_z_dev && c->prm.depth == 1)
            TGV_CUDA(cudaMemsetAsync(grad_v_z_dev, 0, n * 4, s));
        TGV_CUDA(cudaStreamSynchronize(s));  // the scratch is freed on return
        return TGVDCT_OK;
    });
}

tgvdct_status tgvdct_set_pipeline_wait_limit(tgvdct_context* c, uint64_t limit_ns) {
    return guarded([&] {
        TGV_REQUIRE(c != nullptr, "null context");
        c->st.wait_ns = limit_ns;
        if (c->plan) c->plan->wait_ns = limit_ns;
        // the loop and backward graphs hold the old limit in their kernel arguments
        drop_loop_graphs(c);
        if (c->bwd_graph) {
            cudaGraphExecDestroy(c->bwd_graph);
            c->bwd_graph = nullptr;
        }
        return TGVDCT_OK;
    });
}

tgvdct_status tgvdct_check_device_error(tgvdct_context* c, void* stream) {
    return guarded([&] {
        TGV_REQUIRE(c != nullptr, "null context");
        check_tgv_flag(c, (cudaStream_t)stream);
        if (c->plan && !dct_tc_check(c->plan, (cudaStream_t)stream)) {
            set_error("a tensor-core DCT pass timed out waiting on its pipeline");
            return TGVDCT_ERR_TIMEOUT;
        }
        TGV_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
        return TGVDCT_OK;
    });
}

tgvdct_status tgvdct_deshade_epilogue_dev(const float* u_dev, float* l_dev, const float* mask_dev,
                                          uint64_t voxel_count, int32_t mask_shading,
                                          int32_t set_negative_values_to_zero,
                                          int32_t add_background_back, float* r_dev,
                                          void* stream) {
    return guarded([&] {
        TGV_REQUIRE(u_dev && l_dev && r_dev, "null device buffer");
        deshade_epilogue(u_dev, l_dev, mask_dev, (size_t)voxel_count, mask_shading != 0,
                         set_negative_values_to_zero != 0, add_background_back != 0, r_dev,
                         (cudaStream_t)stream);
        return TGVDCT_OK;
    });
}

tgvdct_status tgvdct_process_dev(tgvdct_context* c, const float* f_dev, const float* mask_dev,
                                 int32_t set_negative_values_to_zero, int32_t add_background_back,
                                 int32_t log_domain, float* u_dev, float* l_dev, float* r_dev,
                                 tgvdct_iteration_callback callback, void* user, void* stream) {
    return guarded([&] {
        TGV_REQUIRE(c != nullptr, "null context");
        TGV_REQUIRE(f_dev && u_dev && l_dev && r_dev, "null device buffer");
        TGV_REQUIRE(!(c->domain && mask_dev),
                    "a context with a domain mask uses it in the epilogue; pass mask_dev = NULL");
        process_on_device(c, f_dev, mask_dev, set_negative_values_to_zero != 0,
                          add_background_back != 0, log_domain != 0, u_dev, l_dev, r_dev, callback,
                          user, (cudaStream_t)stream);
        return c->iterations_run < c->prm.iteration_count ? TGVDCT_STOPPED : TGVDCT_OK;
    });
}

tgvdct_status tgvdct_set_domain_mask_dev(tgvdct_context* c, const float* mask_dev, void* stream) {
    return guarded([&] {
        TGV_REQUIRE(c != nullptr, "null context");
        set_domain(c, mask_dev, (cudaStream_t)stream);
        return TGVDCT_OK;
    });
}

tgvdct_status tgvdct_process_tgv2_l1_masked(const tgvdct_params* p, const float* f_host,
                                            const float* mask_host,
                                            int32_t set_negative_values_to_zero,
                                            int32_t add_background_back, int32_t log_domain,
                                            tgvdct_iteration_callback callback, void* user,
                                            float* denoised_host, float* shading_host,
                                            float* deshaded_host) {
    return guarded([&] {
        TGV_REQUIRE(p && f_host && mask_host && denoised_host && shading_host && deshaded_host,
                    "null host buffer");
        tgvdct_params q = *p;
        if (q.depth == 1) q.geometry = TGVDCT_GEOMETRY_2D;  // TGVDeshadeMaskedProcessor.cpp:94-99
        validate(&q);
        HostLease g(q, HK_PROCESS_MASKED, 5);
        tgvdct_context* c = g.c;
        const size_t n = voxels(q);
        float *f = g.buf(0), *m = g.buf(1), *u = g.buf(2), *l = g.buf(3), *r = g.buf(4);
        cudaStream_t s = 0;
        TGV_CUDA(cudaMemcpyAsync(f, f_host, n * 4, cudaMemcpyHostToDevice, s));
        TGV_CUDA(cudaMemcpyAsync(m, mask_host, n * 4, cudaMemcpyHostToDevice, s));
        set_domain(c, m, s);
        process_on_device(c, f, nullptr, set_negative_values_to_zero != 0,
                          add_background_back != 0, log_domain != 0, u, l, r, callback, user, s);
        TGV_CUDA(cudaMemcpyAsync(denoised_host, u, n * 4, cudaMemcpyDeviceToHost, s));
        TGV_CUDA(cudaMemcpyAsync(shading_host, l, n * 4, cudaMemcpyDeviceToHost, s));
        TGV_CUDA(cudaMemcpyAsync(deshaded_host, r, n * 4, cudaMemcpyDeviceToHost, s));
        check_tgv_flag(c, s);
        g.commit();
        return c->iterations_run < q.iteration_count ? TGVDCT_STOPPED : TGVDCT_OK;
    });
}

tgvdct_status tgvdct_tgv2_l1_deshade_masked_launch(
    const float* f_host, const float* mask_host, uint32_t width, uint32_t height, uint32_t depth,
    float lambda, uint32_t iteration_count, uint32_t paint_iteration_interval,
    int cuda_block_dimension, tgvdct_iteration_callback callback, void* user, float alpha0,
    float alpha1, float* u_host, float* v_x_host, float* v_y_host, float* v_z_host) {
    (void)cuda_block_dimension;
    return guarded([&] {
        TGV_REQUIRE(f_host && mask_host && u_host && v_x_host && v_y_host, "null host buffer");
        tgvdct_params p;
        tgvdct_params_init(&p);
        p.width = width;
        p.height = height;
        p.depth = depth;
        p.lambda = lambda;
        p.alpha0 = alpha0;
        p.alpha1 = alpha1;
        p.iteration_count = iteration_count;
        p.paint_iteration_interval = paint_iteration_interval;
        if (depth == 1) p.geometry = TGVDCT_GEOMETRY_2D;
        validate(&p);
        HostLease g(p, HK_DESHADE_MASKED_LAUNCH, 1);
        tgvdct_context* c = g.c;
        const size_t n = voxels(p);
        float* m = g.buf(0);
        cudaStream_t s = 0;
        TGV_CUDA(cudaMemcpyAsync(c->st.f, f_host, n * 4, cudaMemcpyHostToDevice, s));
        TGV_CUDA(cudaMemcpyAsync(m, mask_host, n * 4, cudaMemcpyHostToDevice, s));
        set_domain(c, m, s);
        const bool stopped = run_loop(c, s, callback != nullptr, [&](uint32_t it) {
            return deliver(c, callback, user, it, c->st.u, c->st.v[0], c->st.v[1],
                           c->st.three ? c->st.v[2] : nullptr, s) != 0;
        });
        TGV_CUDA(cudaMemcpyAsync(u_host, c->st.u, n * 4, cudaMemcpyDeviceToHost, s));
        TGV_CUDA(cudaMemcpyAsync(v_x_host, c->st.v[0], n * 4, cudaMemcpyDeviceToHost, s));
        TGV_CUDA(cudaMemcpyAsync(v_y_host, c->st.v[1], n * 4, cudaMemcpyDeviceToHost, s));
        if (v_z_host) {
            if (c->st.three)
                TGV_CUDA(cudaMemcpyAsync(v_z_host, c->st.v[2], n * 4, cudaMemcpyDeviceToHost, s));
            else
                std::memset(v_z_host, 0, n * 4);
        }
        check_tgv_flag(c, s);
        g.commit();
        return stopped ? TGVDCT_STOPPED : TGVDCT_OK;
    });
}

tgvdct_status tgvdct_convergence_test(const tgvdct_params* p, const float* f_host,
                                      const float* mask_host, uint32_t check_iteration_interval,
                                      double* ncc_history, double* time_tv_history,
                                      uint32_t capacity, uint32_t* history_count,
                                      double* metric_tv) {
    return guarded([&] {
        TGV_REQUIRE(p && f_host && metric_tv, "null argument");
        TGV_REQUIRE(check_iteration_interval >= 1, "check_iteration_interval must be >= 1");
        TGV_REQUIRE(capacity == 0 || (ncc_history && time_tv_history), "null history buffer");
        CtxGuard g;
        create_into(p, &g.c);
        tgvdct_context* c = g.c;
        const size_t n = voxels(*p);
        DevBuf m(mask_host ? n : 0);
        cudaStream_t s = 0;
        TGV_CUDA(cudaMemcpyAsync(c->st.f, f_host, n * 4, cudaMemcpyHostToDevice, s));
        if (mask_host) TGV_CUDA(cudaMemcpyAsync(m.p, mask_host, n * 4, cudaMemcpyHostToDevice, s));
        std::vector<double> ncc, tv;
        convergence_on_context(c, mask_host ? m.p : nullptr, check_iteration_interval, ncc, tv,
                               metric_tv, s);
        check_tgv_flag(c, s);
        const size_t k = std::min<size_t>(ncc.size(), capacity);
        for (size_t i = 0; i < k; ++i) {
            ncc_history[i] = ncc[i];
            time_tv_history[i] = tv[i];
        }
        if (history_count) *history_count = (uint32_t)ncc.size();
        return TGVDCT_OK;
    });
}

tgvdct_status tgvdct_convergence_optimization(const tgvdct_params* p, const float* f_host,
                                              const float* mask_host,
                                              int32_t set_negative_values_to_zero,
                                              float* alpha0_out, float* alpha1_out,
                                              float* denoised_host, float* shading_host,
                                              float* deshaded_host) {
    return guarded([&] {
        TGV_REQUIRE(p && f_host && alpha0_out && alpha1_out && denoised_host && shading_host &&
                        deshaded_host,
                    "null argument");
        tgvdct_params q = *p;
        q.iteration_count = 10;  // check_iteration_count (TGVDeshadeProcessor.cpp:583)
        q.paint_iteration_interval = 1;
        CtxGuard g;
        create_into(&q, &g.c);
        tgvdct_context* c = g.c;
        const size_t n = voxels(q);
        DevBuf f(n), m(mask_host ? n : 0);
        cudaStream_t s = 0;
        TGV_CUDA(cudaMemcpyAsync(f.p, f_host, n * 4, cudaMemcpyHostToDevice, s));
        if (mask_host) TGV_CUDA(cudaMemcpyAsync(m.p, mask_host, n * 4, cudaMemcpyHostToDevice, s));
        const float* mask_dev = mask_host ? m.p : nullptr;
        auto metric = [&](double a0, double a1, int which) {
            c->prm.alpha0 = (float)a0;
            c->prm.alpha1 = (float)a1;
            c->prm.iteration_count = 10;
            TGV_CUDA(cudaMemcpyAsync(c->st.f, f.p, n * 4, cudaMemcpyDeviceToDevice, s));
            std::vector<double> ncc, tv;
            double mt[2];
            convergence_on_context(c, mask_dev, 1, ncc, tv, mt, s);
            return (float)mt[which];  // the reference keeps metrics as float
        };
        // decade of alpha1 = alpha0 (:587-612): the first decade whose NCC-series TV
        // falls below the previous one ends the search
        int converged = 0;
        float before = 0.f;
        for (int i = 0; i < 11; ++i) {
            const double a = std::pow(10.0, -i);
            const float v = metric(a, a, 0);
            if (v < before) {
                converged = i - 1;
                break;
            }
            before = v;
        }
        const double alpha1 = std::pow(10.0, -converged);
        // ratio alpha0 / alpha1 maximising the time-TV series' TV (:614-632)
        const double ratios[9] = {1, 1.5, 1.8, 2, 2.2, 2.3, 2.35, 2.4, 2.45};
        int best = 0;
        float best_v = 0.f;
        for (int i = 0; i < 9; ++i) {
            const float v = metric(alpha1 * ratios[i], alpha1, 1);
            if (v > best_v) {
                best_v = v;
                best = i;
            }
        }
        const double alpha0 = ratios[best] * alpha1;
        *alpha0_out = (float)alpha0;
        *alpha1_out = (float)alpha1;
        // the final deshade (:638-645): 500 iterations, the terminal program's overload
        // of processTGV2L1GPUCuda (r weighted by the mask, l not; :122-166)
        c->prm.alpha0 = (float)alpha0;
        c->prm.alpha1 = (float)alpha1;
        c->prm.iteration_count = 500;
        c->prm.paint_iteration_interval = 0;
        TGV_CUDA(cudaMemcpyAsync(c->st.f, f.p, n * 4, cudaMemcpyDeviceToDevice, s));
        run_loop(c, s, false, [](uint32_t) { return false; });
        DevBuf l(n), r(n);
        DctPlan* plan = plan_of(c);
        poisson_integrate(plan, c->st.v[0], c->st.v[1], c->st.three ? c->st.v[2] : nullptr, l.p,
                          c->prm.dct_mode, c->prm.poisson_eigen, s);
        deshade_epilogue(c->st.u, l.p, mask_dev, n, false, set_negative_values_to_zero != 0, false,
                         r.p, s);
        TGV_CUDA(cudaMemcpyAsync(denoised_host, c->st.u, n * 4, cudaMemcpyDeviceToHost, s));
        TGV_CUDA(cudaMemcpyAsync(shading_host, l.p, n * 4, cudaMemcpyDeviceToHost, s));
        TGV_CUDA(cudaMemcpyAsync(deshaded_host, r.p, n * 4, cudaMemcpyDeviceToHost, s));
        check_tgv_flag(c, s);
        return TGVDCT_OK;
    });
}

tgvdct_status tgvdct_process_tgv2_l1(const tgvdct_params* p, const float* f_host,
                                     const float* mask_host, int32_t set_negative_values_to_zero,
                                     int32_t add_background_back, int32_t log_domain,
                                     tgvdct_iteration_callback callback, void* user,
                                     float* denoised_host, float* shading_host,
                                     float* deshaded_host) {
    return guarded([&] {
        TGV_REQUIRE(f_host && denoised_host && shading_host && deshaded_host, "null host buffer");
        validate(p);
        HostLease g(*p, HK_PROCESS, mask_host ? 5 : 4);
        tgvdct_context* c = g.c;
        const size_t n = voxels(*p);
        float *f = g.buf(0), *u = g.buf(1), *l = g.buf(2), *r = g.buf(3);
        float* m = mask_host ? g.buf(4) : nullptr;
        cudaStream_t s = 0;
        TGV_CUDA(cudaMemcpyAsync(f, f_host, n * 4, cudaMemcpyHostToDevice, s));
        if (mask_host) TGV_CUDA(cudaMemcpyAsync(m, mask_host, n * 4, cudaMemcpyHostToDevice, s));
        process_on_device(c, f, m, set_negative_values_to_zero != 0, add_background_back != 0,
                          log_domain != 0, u, l, r, callback, user, s);
        TGV_CUDA(cudaMemcpyAsync(denoised_host, u, n * 4, cudaMemcpyDeviceToHost, s));
        TGV_CUDA(cudaMemcpyAsync(shading_host, l, n * 4, cudaMemcpyDeviceToHost, s));
        TGV_CUDA(cudaMemcpyAsync(deshaded_host, r, n * 4, cudaMemcpyDeviceToHost, s));
        check_tgv_flag(c, s);
        if (c->plan && !dct_tc_check(c->plan, s)) {
            set_error("a tensor-core DCT pass timed out waiting on its pipeline");
            return TGVDCT_ERR_TIMEOUT;
        }
        g.commit();
        return c->iterations_run < p->iteration_count ? TGVDCT_STOPPED : TGVDCT_OK;
    });
}

tgvdct_status tgvdct_release_cached(void) {
    return guarded([&] {
        CacheClaim claim;
        TGV_REQUIRE(claim.owned, "the cached context is in use by a running call");
        host_cache_drop(host_cache());
        return TGVDCT_OK;
    });
}

tgvdct_status tgvdct_resize_bspline3_dev(const float* in_dev, uint32_t width, uint32_t height,
                                         uint32_t depth, float* out_dev, uint32_t out_width,
                                         uint32_t out_height, uint32_t out_depth, void* stream) {
    return guarded([&] {
        TGV_REQUIRE(in_dev && out_dev, "null device buffer");
        TGV_REQUIRE(width >= 1 && height >= 1 && depth >= 1 && out_width >= 1 &&
                        out_height >= 1 && out_depth >= 1,
                    "extents must be >= 1");
        check_device();
        cudaStream_t s = (cudaStream_t)stream;
        DevBuf scratch((resize_scratch_bytes((int)width, (int)height, (int)depth, (int)out_width,
                                             (int)out_height, (int)out_depth) +
                        3) /
                       4);
        resize_bspline3(in_dev, (int)width, (int)height, (int)depth, out_dev, (int)out_width,
                        (int)out_height, (int)out_depth, scratch.p, s);
        TGV_CUDA(cudaStreamSynchronize(s));
        return TGVDCT_OK;
    });
}

tgvdct_status tgvdct_resize_bspline3(const float* in_host, uint32_t width, uint32_t height,
                                     uint32_t depth, float* out_host, uint32_t out_width,
                                     uint32_t out_height, uint32_t out_depth) {
    return guarded([&] {
        TGV_REQUIRE(in_host && out_host, "null host buffer");
        TGV_REQUIRE(width >= 1 && height >= 1 && depth >= 1 && out_width >= 1 &&
                        out_height >= 1 && out_depth >= 1,
                    "extents must be >= 1");
        check_device();
        const size_t n = (size_t)width * height * depth;
        const size_t m = (size_t)out_width * out_height * out_depth;
        DevBuf a(n), b(m);
        DevBuf scratch((resize_scratch_bytes((int)width, (int)height, (int)depth, (int)out_width,
                                             (int)out_height, (int)out_depth) +
                        3) /
                       4);
        TGV_CUDA(cudaMemcpy(a.p, in_host, n * 4, cudaMemcpyHostToDevice));
        resize_bspline3(a.p, (int)width, (int)height, (int)depth, b.p, (int)out_width,
                        (int)out_height, (int)out_depth, scratch.p, 0);
        TGV_CUDA(cudaMemcpy(out_host, b.p, m * 4, cudaMemcpyDeviceToHost));
        return TGVDCT_OK;
    });
}

uint32_t tgvdct_resize_factor_extent(uint32_t n, float factor) {
    return resize_factor_extent(n, factor);
}

namespace {
void check_downsampled_args(uint32_t width, uint32_t height, uint32_t depth, float factor,
                            uint32_t order, const float* alpha) {
    TGV_REQUIRE(width >= 1 && height >= 1 && depth >= 1, "width, height, depth must be >= 1");
    TGV_REQUIRE(factor > 0.f, "downsampling_factor must be > 0");
    TGV_REQUIRE(alpha != nullptr, "null alpha array");
    if (order != 2) {
        set_error("order " + std::to_string(order) +
                  ": only order 2 is built (the reference runs its TGV2 processors for it); "
                  "TGVk of other orders is not part of this library");
        throw Error{TGVDCT_ERR_UNSUPPORTED};
    }
}
}  // namespace

tgvdct_status tgvdct_process_tgvk_l1_downsampled_dev(
    const float* f_dev, const float* mask_dev, uint32_t width, uint32_t height, uint32_t depth,
    float downsampling_factor, float lambda, uint32_t order, const float* alpha,
    uint32_t iteration_count, int32_t set_negative_values_to_zero, int32_t add_background_back,
    int32_t not_masked, uint32_t paint_iteration_interval, tgvdct_iteration_callback callback,
    void* user, float* denoised_dev, float* shading_dev, float* deshaded_dev, float* div_v_dev,
    void* stream) {
    return guarded([&] {
        TGV_REQUIRE(f_dev && denoised_dev && shading_dev && deshaded_dev, "null device buffer");
        check_downsampled_args(width, height, depth, downsampling_factor, order, alpha);
        check_device();
        const bool stopped = downsampled_on_device(
            f_dev, mask_dev, width, height, depth, downsampling_factor, lambda, alpha,
            iteration_count, paint_iteration_interval, set_negative_values_to_zero != 0,
            add_background_back != 0, not_masked != 0, callback, user, denoised_dev, shading_dev,
            deshaded_dev, div_v_dev, (cudaStream_t)stream);
        return stopped ? TGVDCT_STOPPED : TGVDCT_OK;
    });
}

tgvdct_status tgvdct_process_tgvk_l1_downsampled(
    const float* f_host, const float* mask_host, uint32_t width, uint32_t height, uint32_t depth,
    float downsampling_factor, float lambda, uint32_t order, const float* alpha,
    uint32_t iteration_count, int32_t set_negative_values_to_zero, int32_t add_background_back,
    int32_t not_masked, uint32_t paint_iteration_interval, tgvdct_iteration_callback callback,
    void* user, float* denoised_host, float* shading_host, float* deshaded_host,
    float* div_v_host) {
    return guarded([&] {
        TGV_REQUIRE(f_host && denoised_host && shading_host && deshaded_host, "null host buffer");
        check_downsampled_args(width, height, depth, downsampling_factor, order, alpha);
        check_device();
        const size_t n = (size_t)width * height * depth;
        DevBuf f(n), m(mask_host ? n : 0), u(n), l(n), r(n), dv(div_v_host ? n : 0);
        TGV_CUDA(cudaMemcpy(f.p, f_host, n * 4, cudaMemcpyHostToDevice));
        if (mask_host) TGV_CUDA(cudaMemcpy(m.p, mask_host, n * 4, cudaMemcpyHostToDevice));
        const bool stopped = downsampled_on_device(
            f.p, mask_host ? m.p : nullptr, width, height, depth, downsampling_factor, lambda,
            alpha, iteration_count, paint_iteration_interval, set_negative_values_to_zero != 0,
            add_background_back != 0, not_masked != 0, callback, user, u.p, l.p, r.p,
            div_v_host ? dv.p : nullptr, 0);
        TGV_CUDA(cudaMemcpy(denoised_host, u.p, n * 4, cudaMemcpyDeviceToHost));
        TGV_CUDA(cudaMemcpy(shading_host, l.p, n * 4, cudaMemcpyDeviceToHost));
        TGV_CUDA(cudaMemcpy(deshaded_host, r.p, n * 4, cudaMemcpyDeviceToHost));
        if (div_v_host) TGV_CUDA(cudaMemcpy(div_v_host, dv.p, n * 4, cudaMemcpyDeviceToHost));
        return stopped ? TGVDCT_STOPPED : TGVDCT_OK;
    });
}

namespace {
void check_energy_args(const tgvdct_params* p) {
    validate(p);
    TGV_REQUIRE(p->lambda >= 0.f && p->alpha0 >= 0.f && p->alpha1 >= 0.f,
                "energy weights must be >= 0");
}
bool energy_three(const tgvdct_params* p) { return p->geometry != TGVDCT_GEOMETRY_2D; }
}  // namespace

tgvdct_status tgvdct_tgv2_energy_dev(const tgvdct_params* p, const float* f_dev,
                                     const float* u_dev, const float* v_x_dev,
                                     const float* v_y_dev, const float* v_z_dev,
                                     double* energy_dev, void* stream) {
    return guarded([&] {
        check_energy_args(p);
        const bool three = energy_three(p);
        TGV_REQUIRE(f_dev && u_dev && v_x_dev && v_y_dev && (v_z_dev || !three) && energy_dev,
                    "null device buffer");
        check_device();
        tgv_energy_terms(f_dev, u_dev, v_x_dev, v_y_dev, three ? v_z_dev : nullptr,
                         (int)p->width, (int)p->height, (int)p->depth, three, p->data_term,
                         energy_dev, (cudaStream_t)stream);
        return TGVDCT_OK;
    });
}

tgvdct_status tgvdct_tgv2_energy(const tgvdct_params* p, const float* f_host,
                                 const float* u_host, const float* v_x_host,
                                 const float* v_y_host, const float* v_z_host, double* energy) {
    return guarded([&] {
        check_energy_args(p);
        const bool three = energy_three(p);
        TGV_REQUIRE(f_host && u_host && v_x_host && v_y_host && (v_z_host || !three) && energy,
                    "null host buffer");
        check_device();
        const size_t n = voxels(*p);
        DevBuf f(n), u(n), vx(n), vy(n), vz(three ? n : 0), sums(2 * 3);
        TGV_CUDA(cudaMemcpy(f.p, f_host, n * 4, cudaMemcpyHostToDevice));
        TGV_CUDA(cudaMemcpy(u.p, u_host, n * 4, cudaMemcpyHostToDevice));
        TGV_CUDA(cudaMemcpy(vx.p, v_x_host, n * 4, cudaMemcpyHostToDevice));
        TGV_CUDA(cudaMemcpy(vy.p, v_y_host, n * 4, cudaMemcpyHostToDevice));
        if (three) TGV_CUDA(cudaMemcpy(vz.p, v_z_host, n * 4, cudaMemcpyHostToDevice));
        double* d = (double*)sums.p;
        tgv_energy_terms(f.p, u.p, vx.p, vy.p, three ? vz.p : nullptr, (int)p->width,
                         (int)p->height, (int)p->depth, three, p->data_term, d, 0);
        double h[3];
        TGV_CUDA(cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost));
        energy[0] = (double)p->lambda * h[0];
        energy[1] = (double)p->alpha1 * h[1];
        energy[2] = (double)p->alpha0 * h[2];
        energy[3] = energy[0] + energy[1] + energy[2];
        return TGVDCT_OK;
    });
}

tgvdct_status tgvdct_energy_history(tgvdct_context* c, double* out, uint32_t capacity,
                                    uint32_t* count) {
    return guarded([&] {
        TGV_REQUIRE(c != nullptr, "null context");
        TGV_REQUIRE(count != nullptr && (out != nullptr || capacity == 0), "null output");
        const size_t m = c->energy_history.size();
        *count = (uint32_t)m;
        for (size_t i = 0; i < m && i < capacity; ++i) out[i] = c->energy_history[i];
        return TGVDCT_OK;
    });
}

tgvdct_status tgvdct_request_stop(tgvdct_context* c) {
    if (!c) {
        tgvdct::set_error("null context");
        return TGVDCT_ERR_BAD_ARG;
    }
    c->stop_requested.store(true);
    return TGVDCT_OK;
}

tgvdct_status tgvdct_bounds_check(uint64_t* first_bad) {
    return guarded([&]() -> tgvdct_status {
        TGV_REQUIRE(first_bad != nullptr, "null output");
        if constexpr (kCheckBounds) {
            TGV_CUDA(cudaDeviceSynchronize());
            const uint64_t w[3] = {tgv_kernels_bounds_take(), adjoint_bounds_take(),
                                   resize_bounds_take()};
            *first_bad = w[0] ? w[0] : w[1] ? w[1] : w[2];
            return TGVDCT_OK;
        } else {
            set_error("this library is built without bounds checks (libtgvdct_checked.so has them)");
            throw Error{TGVDCT_ERR_UNSUPPORTED};
        }
    });
}

}  // extern "C"
