// Host driver of the GB300 bundle adjuster and the C ABI (include/sfmba.h).
//
// The Levenberg-Marquardt loop follows crates/sfm-ba/src/lib.rs:747-1232:
// slots for free poses then free cameras; per outer iteration one
// linearisation; up to 8 damping retries, each building the reduced system,
// solving it, back-substituting the points and evaluating the trial cost;
// accept iff the FP64 trial cost is finite and lower; stop when no retry is
// accepted or the relative decrease drops below 1e-6. Damping, acceptance
// and all parameters live on the device; the host reads a 100-byte state
// record once per retry to decide whether to launch another one.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include <cub/cub.cuh>

#include "camera.cuh"
#include "colmap_io.h"
#include "kernels.cuh"
#include "ozaki.cuh"

namespace sfmba {

thread_local long long g_kernel_launches = 0;

namespace {

constexpr int kPcgPollEvery = 8;  // PCG iterations between host convergence polls
constexpr int kDenseMaxDim = 16384;  // largest reduced system the dense path forms

thread_local std::string g_last_error;

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}


// Per-phase device timing: CUDA events on the launch stream around each
// kernel phase, resolved after the solve's final synchronisation.
const char *const kPhaseNames[] = {"setup",        "linearize",   "point_reduce", "image_reduce",
                                   "point_inverse", "image_rhs",  "schur_pairs",  "fold",
                                   "cholesky",     "trsv",        "refine",       "pcg_precond",
                                   "pcg_points",   "pcg_images",  "pcg_vector",   "backsub_update",
                                   "cost",         "lu",          "lm_bookkeeping", "coarse_assemble",
                                   "coarse_factor"};
enum Phase {
    PH_SETUP, PH_LINEARIZE, PH_POINT_REDUCE, PH_IMAGE_REDUCE, PH_POINT_INVERSE, PH_IMAGE_RHS,
    PH_SCHUR, PH_FOLD, PH_CHOLESKY, PH_TRSV, PH_REFINE, PH_PCG_PRECOND, PH_PCG_POINTS,
    PH_PCG_IMAGES, PH_PCG_VECTOR, PH_BACKSUB, PH_COST, PH_LU, PH_LM, PH_COARSE_ASSEMBLE, PH_COARSE_FACTOR,
    PH_COUNT
};

struct Profiler {
    bool on = false;
    std::vector<cudaEvent_t> pool;
    size_t used = 0;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
    double ms[PH_COUNT] = {0};
    long long launches[PH_COUNT] = {0};
    std::map<std::string, double> host_ms;  // wall time of host stages (ms)
    std::map<std::string, long long> counts;  // event counts (coarse inverses, their breakdowns)
    std::vector<std::string> trace;           // one JSON object per LM outer iteration of single solves
    void host(const char *name, double seconds) {
        if (on) host_ms[name] += seconds * 1e3;
    }
    void count(const char *name, long long k) {
        if (on) counts[name] += k;
    }
    cudaEvent_t take() {
        if (used == pool.size()) {
            cudaEvent_t e;
            SFMBA_CUDA(cudaEventCreate(&e));
            pool.push_back(e);
        }
        return pool[used++];
    }
    void resolve() {
        for (auto &p : pending) {
            float t = 0.f;
            if (cudaEventElapsedTime(&t, p.second.first, p.second.second) == cudaSuccess) {
                ms[p.first] += t;
                launches[p.first] += 1;
            } else {
                (void)cudaGetLastError();
            }
        }
        pending.clear();
        used = 0;
    }
    void reset() {
        resolve();
        for (int k = 0; k < PH_COUNT; ++k) { ms[k] = 0; launches[k] = 0; }
        host_ms.clear();
        counts.clear();
        trace.clear();
    }
};

Profiler &profiler() {
    thread_local Profiler p;
    return p;
}

// Wall time of the set-up's stages under the profiler: mark(name) waits for
// the stream and charges the time since the previous mark to name (host
// work, host-device copies and the stage's kernels), so the stages add up
// to the set-up phase. Does nothing when profiling is off.
struct StageClock {
    cudaStream_t s;
    double t;
    explicit StageClock(cudaStream_t stream) : s(stream), t(now_s()) {}
    void mark(const char *name) {
        if (!profiler().on) return;
        SFMBA_CUDA(cudaStreamSynchronize(s));
        const double u = now_s();
        profiler().host(name, u - t);
        t = u;
    }
};

// Brackets the launches of one phase with events when profiling is on.
struct PhaseScope {
    Profiler &p;
    int ph;
    cudaStream_t s;
    cudaEvent_t a = nullptr;
    PhaseScope(int phase, cudaStream_t stream) : p(profiler()), ph(phase), s(stream) {
        if (p.on) {
            a = p.take();
            SFMBA_CUDA(cudaEventRecord(a, s));
        }
    }
    ~PhaseScope() {
        if (p.on && a) {
            cudaEvent_t b = p.take();
            if (cudaEventRecord(b, s) == cudaSuccess) p.pending.push_back({ph, {a, b}});
            else (void)cudaGetLastError();
        }
    }
};
#define SFMBA_PHASE_CAT2(a, b) a##b
#define SFMBA_PHASE_CAT(a, b) SFMBA_PHASE_CAT2(a, b)
#define SFMBA_PHASE(ph) PhaseScope SFMBA_PHASE_CAT(phase_scope_, __LINE__)(ph, s_)

// A launch sequence that repeats with the same arguments (a PCG chunk, a
// batched retry round): run directly the first time, captured from the
// stream the second time, then launched as one CUDA graph. Bypassed while
// the phase profiler is on (its events bracket individual launches) and on
// the legacy default stream (which cannot be captured). The kernel-launch
// counter counts the graph's kernels at every replay.
class Replay {
  public:
    ~Replay() { reset(); }
    void reset() {
        if (exec_) cudaGraphExecDestroy(exec_);
        exec_ = nullptr;
        uses_ = 0;
    }
    template <typename F>
    void run(cudaStream_t s, bool allowed, F &&f) {
        if (!allowed || s == cudaStreamLegacy || uses_++ == 0) {
            f();
            return;
        }
        if (!exec_) {
            const long long before = g_kernel_launches;
            SFMBA_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
            try {
                f();
            } catch (...) {
                cudaGraph_t tmp = nullptr;
                cudaStreamEndCapture(s, &tmp);
                if (tmp) cudaGraphDestroy(tmp);
                (void)cudaGetLastError();
                throw;
            }
            cudaGraph_t g = nullptr;
            SFMBA_CUDA(cudaStreamEndCapture(s, &g));
            kernels_ = g_kernel_launches - before;
            g_kernel_launches = before;
            const cudaError_t e = cudaGraphInstantiate(&exec_, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) exec_ = nullptr;
            SFMBA_CUDA(e);
        }
        SFMBA_CUDA(cudaGraphLaunch(exec_, s));
        g_kernel_launches += kernels_;
    }

  private:
    cudaGraphExec_t exec_ = nullptr;
    long long kernels_ = 0;
    int uses_ = 0;
};

// Bump allocator over one device allocation that grows on demand and is
// kept across calls on the same thread.
class Arena {
  public:
    ~Arena() { release(); }
    void release() {
        if (base_) cudaFree(base_);
        base_ = nullptr;
        cap_ = 0;
    }
    void begin_sizing() { sizing_ = true; off_ = 0; }
    void commit() {
        if (off_ > cap_) {
            release();
            size_t want = off_ + (off_ >> 3) + (1 << 20);
            SFMBA_CUDA(cudaMalloc(&base_, want));
            cap_ = want;
        }
        sizing_ = false;
        off_ = 0;
    }
    template <typename T>
    T *take(size_t count) {
        size_t bytes = ((count * sizeof(T)) + 255) / 256 * 256;
        if (bytes == 0) bytes = 256;
        char *p = sizing_ ? nullptr : base_ + off_;
        off_ += bytes;
        return reinterpret_cast<T *>(p);
    }

  private:
    char *base_ = nullptr;
    size_t cap_ = 0, off_ = 0;
    bool sizing_ = false;
};

// Autotuner of launch variants: the PCG passes (ILP depth, records loaded
// ahead, minimum blocks per SM; mf_passes.cuh) and the batched windows'
// Schur reduction (warps per block, minimum blocks per SM; k_batched.cu).
// Per device, kernel, block width and problem size (log2 of the
// observation count) the variant with the shortest mean of three timed
// launches on a solve's own buffers, measured once at the first use and
// kept for the process. Every variant computes the same sums in the same
// order, so the choice never changes results.
struct TuneEntry {
    int variant = 0;
    int count = 0;  // variants timed
    float us[kPassVariants] = {0};
};
std::mutex g_tune_mu;
std::map<std::tuple<int, int, int, int>, TuneEntry> g_tune;  // (device, pass, D, size bucket)

template <typename Launch>
int tuned_variant(int device, int pass, int count, const Bufs &b, cudaStream_t s, Launch launch) {
    int bucket = 0;
    for (long long n = std::max<long long>(b.nO, 1); n > 1; n >>= 1) ++bucket;
    const auto key = std::make_tuple(device, pass, b.D, bucket);
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_tune.find(key);
    if (it != g_tune.end()) return it->second.variant;
    TuneEntry e;
    e.count = count;
    cudaEvent_t a, z;
    SFMBA_CUDA(cudaEventCreate(&a));
    SFMBA_CUDA(cudaEventCreate(&z));
    float best = 0.f;
    for (int v = 0; v < count; ++v) {
        launch(v);  // warm-up
        SFMBA_CUDA(cudaEventRecord(a, s));
        for (int r = 0; r < 3; ++r) launch(v);
        SFMBA_CUDA(cudaEventRecord(z, s));
        SFMBA_CUDA(cudaEventSynchronize(z));
        float ms = 0.f;
        SFMBA_CUDA(cudaEventElapsedTime(&ms, a, z));
        e.us[v] = ms * 1e3f / 3.f;
        if (v == 0 || e.us[v] < best) {
            best = e.us[v];
            e.variant = v;
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(z);
    g_tune[key] = e;
    return e.variant;
}

std::string tune_report() {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    std::string js = "[";
    bool first = true;
    for (const auto &kv : g_tune) {
        char tmp[256];
        const TuneEntry &e = kv.second;
        std::snprintf(tmp, sizeof(tmp), "%s{\"device\":%d,\"pass\":\"%s\",\"D\":%d,\"log2_obs\":%d,\"variant\":%d,\"us\":[",
                      first ? "" : ",", std::get<0>(kv.first),
                      std::get<1>(kv.first) == 0   ? "points"
                      : std::get<1>(kv.first) == 1 ? "images"
                      : std::get<1>(kv.first) == 2 ? "wb_schur"
                                                   : "wb_schur_fp64",
                      std::get<2>(kv.first), std::get<3>(kv.first), e.variant);
        js += tmp;
        for (int v = 0; v < e.count; ++v) {
            std::snprintf(tmp, sizeof(tmp), "%s%.2f", v ? "," : "", e.us[v]);
            js += tmp;
        }
        js += "]}";
        first = false;
    }
    return js + "]";
}

struct Context {
    int device = -1;
    cudaStream_t stream = nullptr;
    Arena main, pairs, aux, coarse, shared, shared_inc;
    LMState *h_state = nullptr;  // pinned mirror
    int *h_counts = nullptr;     // pinned batch summary
    ~Context() {
        if (h_state) cudaFreeHost(h_state);
        if (h_counts) cudaFreeHost(h_counts);
        if (stream) cudaStreamDestroy(stream);
    }
};

Context &context() {
    thread_local std::unique_ptr<Context> ctx;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        throw Error(SFMBA_ERR_NO_DEVICE, std::string("no CUDA device: ") + cudaGetErrorString(e));
    }
    int count = 0;
    e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        (void)cudaGetLastError();
        throw Error(SFMBA_ERR_NO_DEVICE, "no CUDA device available");
    }
    if (!ctx || ctx->device != dev) {
        ctx.reset(new Context());
        ctx->device = dev;
        SFMBA_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
        SFMBA_CUDA(cudaMallocHost(&ctx->h_state, sizeof(LMState)));
        SFMBA_CUDA(cudaMallocHost(&ctx->h_counts, 4 * sizeof(int)));
    }
    return *ctx;
}

// Host view of the slot structure (lib.rs:753-776) and the image blocks.
struct Layout {
    int nI = 0, nC = 0, nP = 0;
    long long nO = 0;
    int n = 0, D = 6;
    std::vector<int> pose_slot, cam_slot, img_slot, img_active, img_free;
    std::vector<int> slot_pre_start, slot_pre;
    std::vector<unsigned char> slot_masked;
    bool injective = true;
    // Free cameras used by several images (PCG solver, k_shared.cu): the
    // owner image (first user) of each image's camera columns, its shared-
    // camera index, the column masks of the PCG vector kernels, and the
    // images of each shared camera in image order.
    std::vector<int> img_owner, img_shcam, img_pmask, img_dmask;
    std::vector<int> sh_img_start, sh_imgs;
};

Layout make_layout(int nI, int nC, int nP, long long nO, const std::vector<int> &cam_of_img,
                   const std::vector<int> &model, const std::vector<unsigned char> &fixed_pose,
                   const std::vector<unsigned char> &fixed_cam, const std::vector<unsigned char> &fixed_cp,
                   int force_D = 0) {
    Layout L;
    L.nI = nI; L.nC = nC; L.nP = nP; L.nO = nO;
    L.pose_slot.assign(nI, -1);
    L.cam_slot.assign(nC, -1);
    int n = 0;
    for (int i = 0; i < nI; ++i)
        if (!fixed_pose[i]) { L.pose_slot[i] = n; n += 6; }
    int kmax = 0;
    for (int c = 0; c < nC; ++c)
        if (!fixed_cam[c]) {
            L.cam_slot[c] = n;
            n += model_dof(model[c]);
            kmax = std::max(kmax, model_dof(model[c]));
        }
    L.n = n;
    L.D = std::max(block_width_for(kmax), force_D);
    const int D = L.D;
    L.img_slot.assign((size_t)nI * D, -1);
    L.img_active.assign(nI, 0);
    L.img_free.assign(nI, 0);
    L.slot_masked.assign(n, 0);
    for (int c = 0; c < nC; ++c) {
        if (L.cam_slot[c] < 0) continue;
        for (int k = 0; k < model_dof(model[c]); ++k)
            if (fixed_cp[(size_t)c * 8 + k]) L.slot_masked[L.cam_slot[c] + k] = 1;
    }
    // (slot, image block entry) of every image entry that maps to a slot, in
    // image order; grouped by slot below (stable), one allocation for all.
    std::vector<std::pair<int, int>> pre;
    pre.reserve((size_t)n);
    std::vector<int> cam_users(nC, 0);
    for (int i = 0; i < nI; ++i) {
        const int c = cam_of_img[i];
        int act = 0;
        if (L.pose_slot[i] >= 0)
            for (int r = 0; r < 6; ++r) {
                L.img_slot[(size_t)i * D + r] = L.pose_slot[i] + r;
                pre.emplace_back(L.pose_slot[i] + r, i * D + r);
                act |= 1 << r;
            }
        if (L.cam_slot[c] >= 0) {
            cam_users[c] += 1;
            for (int k = 0; k < model_dof(model[c]); ++k) {
                const int slot = L.cam_slot[c] + k;
                if (L.slot_masked[slot]) continue;
                L.img_slot[(size_t)i * D + 6 + k] = slot;
                pre.emplace_back(slot, i * D + 6 + k);
                act |= 1 << (6 + k);
            }
        }
        L.img_active[i] = act;
        L.img_free[i] = (L.pose_slot[i] >= 0 || L.cam_slot[c] >= 0) ? 1 : 0;
    }
    for (int c = 0; c < nC; ++c)
        if (cam_users[c] > 1) L.injective = false;
    L.img_owner.resize(nI);
    L.img_shcam.assign(nI, -1);
    L.img_pmask = L.img_active;
    L.img_dmask = L.img_active;
    std::vector<int> owner(nC, -1), shidx(nC, -1), sh_count;
    for (int i = 0; i < nI; ++i) {
        const int c = cam_of_img[i];
        L.img_owner[i] = i;
        if (L.cam_slot[c] < 0 || cam_users[c] < 2) continue;
        if (owner[c] < 0) {
            owner[c] = i;
            shidx[c] = (int)sh_count.size();
            sh_count.push_back(0);
        }
        L.img_owner[i] = owner[c];
        L.img_shcam[i] = shidx[c];
        sh_count[shidx[c]] += 1;
        L.img_pmask[i] = L.img_active[i] & 0x3f;
        if (owner[c] != i) L.img_dmask[i] = L.img_active[i] & 0x3f;
    }
    const int nsh = (int)sh_count.size();
    L.sh_img_start.assign(nsh + 1, 0);
    for (int k = 0; k < nsh; ++k) L.sh_img_start[k + 1] = L.sh_img_start[k] + sh_count[k];
    L.sh_imgs.resize(L.sh_img_start[nsh]);
    {
        std::vector<int> fill(L.sh_img_start.begin(), L.sh_img_start.end() - 1);
        for (int i = 0; i < nI; ++i)
            if (L.img_shcam[i] >= 0) L.sh_imgs[fill[L.img_shcam[i]]++] = i;
    }
    L.slot_pre_start.assign(n + 1, 0);
    for (const auto &e : pre) L.slot_pre_start[e.first + 1] += 1;
    for (int a = 0; a < n; ++a) L.slot_pre_start[a + 1] += L.slot_pre_start[a];
    L.slot_pre.assign(L.slot_pre_start[n], 0);
    {
        std::vector<int> fill(L.slot_pre_start.begin(), L.slot_pre_start.end() - 1);
        for (const auto &e : pre) L.slot_pre[fill[e.first]++] = e.second;
    }
    return L;
}

// A batch of independent windows concatenated into one problem: images,
// cameras, points and observations in window order, indices offset, and a
// slot layout that keeps each window's unknowns contiguous (each window
// slotted as its own problem, lib.rs:753-776), with one image block width
// for the whole batch.
struct Batch {
    int W = 0;
    Layout lay;
    int max_n = 0;
    std::vector<int> img_base, cam_base, pt_base, slot_base, n_w, nid_w;
    std::vector<long long> obs_off, s_off, simg_off, linv_off;
    long long s_total = 0, simg_total = 0, linv_total = 0;
    std::vector<int> img_win, cam_win, slot_win, win_of_point;
    std::vector<int> slot_perm;  // position in the window systems -> slot (global)
    std::vector<int> cblk_win, wblk_start;  // cost blocks (kWinCostChunk observations)
    std::vector<int4> fold_blk;             // fold blocks: {window, first row, end row}
    std::vector<long long> cblk_lo;
    // concatenated problem arrays
    std::vector<int> cam_of_img, model, obs_image, obs_point;
    std::vector<double> cams, poses, points, obs_xy;
    std::vector<unsigned char> fixed_pose, fixed_cam, fixed_cp;
    sfmba_problem problem{};
    const sfmba_problem *windows = nullptr;
    const sfmba_problem &window(int w) const { return windows[w]; }
};

// Runs f(k) for k in [0, n) on up to 16 host threads, in contiguous ranges.
template <typename F>
void parallel_for(int n, F &&f) {
    const int threads = std::max(1, std::min<int>({16, (int)std::thread::hardware_concurrency(), n}));
    if (threads <= 1) {
        for (int k = 0; k < n; ++k) f(k);
        return;
    }
    std::vector<std::thread> pool;
    std::exception_ptr err;
    std::mutex mu;
    for (int t = 0; t < threads; ++t)
        pool.emplace_back([&, t] {
            try {
                for (int k = (int)((long long)n * t / threads); k < (int)((long long)n * (t + 1) / threads); ++k) f(k);
            } catch (...) {
                std::lock_guard<std::mutex> lock(mu);
                if (!err) err = std::current_exception();
            }
        });
    for (auto &th : pool) th.join();
    if (err) std::rethrow_exception(err);
}

void build_batch(int W, const sfmba_problem *win, Batch &B) {
    // the window index is a grid dimension (y or z) of the per-window kernels
    if (W > 65535) throw Error(SFMBA_ERR_UNSUPPORTED, "at most 65535 windows per batch");
    B.W = W;
    B.windows = win;
    long long nI = 0, nC = 0, nP = 0, nO = 0;
    int kmax = 0;
    for (int w = 0; w < W; ++w) {
        const sfmba_problem &p = win[w];
        for (long long c = 0; c < p.num_cameras; ++c)
            if (!(p.fixed_cameras && p.fixed_cameras[c])) kmax = std::max(kmax, model_dof(p.camera_model[c]));
        nI += p.num_images; nC += p.num_cameras; nP += p.num_points; nO += p.num_observations;
    }
    if (nI > 65535) throw Error(SFMBA_ERR_UNSUPPORTED, "batched solve supports at most 65535 images in total");
    if (nC > (1 << 20) || nP > (1LL << 30) || nO > (1LL << 31) - 1)
        throw Error(SFMBA_ERR_INVALID_ARGUMENT, "batch too large for 32-bit indices");
    const int D = block_width_for(kmax);
    Layout &L = B.lay;
    L.nI = (int)nI; L.nC = (int)nC; L.nP = (int)nP; L.nO = nO; L.D = D;
    B.img_base.resize(W); B.cam_base.resize(W); B.pt_base.resize(W); B.slot_base.resize(W);
    B.n_w.resize(W); B.nid_w.resize(W);
    B.obs_off.assign(W + 1, 0); B.s_off.resize(W); B.simg_off.resize(W); B.linv_off.resize(W);
    B.cam_of_img.reserve(nI); B.model.reserve(nC);
    B.cams.reserve(nC * 8); B.poses.reserve(nI * 7);
    B.fixed_pose.reserve(nI); B.fixed_cam.reserve(nC); B.fixed_cp.reserve(nC * 8);
    B.img_win.reserve(nI); B.cam_win.reserve(nC);
    int ib = 0, cb = 0, pb = 0, sb = 0;
    long long ob = 0, so = 0, sio = 0, lo = 0;
    // Each window slotted on its own (independent), on the host threads.
    std::vector<Layout> lays(W);
    parallel_for(W, [&](int w) {
        const sfmba_problem &p = win[w];
        const int wi = (int)p.num_images, wc = (int)p.num_cameras;
        std::vector<int> coi(p.camera_of_image, p.camera_of_image + wi);
        std::vector<int> mod(p.camera_model, p.camera_model + wc);
        std::vector<unsigned char> fp(wi, 0), fc(wc, 0), fcp((size_t)wc * 8, 0);
        if (p.fixed_poses) fp.assign(p.fixed_poses, p.fixed_poses + wi);
        if (p.fixed_cameras) fc.assign(p.fixed_cameras, p.fixed_cameras + wc);
        if (p.fixed_camera_params) fcp.assign(p.fixed_camera_params, p.fixed_camera_params + (size_t)wc * 8);
        lays[w] = make_layout(wi, wc, (int)p.num_points, p.num_observations, coi, mod, fp, fc, fcp, D);
    });
    for (int w = 0; w < W; ++w) {
        const sfmba_problem &p = win[w];
        const int wi = (int)p.num_images, wc = (int)p.num_cameras, wp = (int)p.num_points;
        const long long wo = p.num_observations;
        const int *coi = p.camera_of_image, *mod = p.camera_model;
        std::vector<unsigned char> fp(wi, 0), fc(wc, 0), fcp((size_t)wc * 8, 0);
        if (p.fixed_poses) fp.assign(p.fixed_poses, p.fixed_poses + wi);
        if (p.fixed_cameras) fc.assign(p.fixed_cameras, p.fixed_cameras + wc);
        if (p.fixed_camera_params) fcp.assign(p.fixed_camera_params, p.fixed_camera_params + (size_t)wc * 8);
        const Layout &lw = lays[w];
        if (lw.n > 16384)
            throw Error(SFMBA_ERR_UNSUPPORTED, "window " + std::to_string(w) + " has more than 16384 unknowns");
        B.img_base[w] = ib; B.cam_base[w] = cb; B.pt_base[w] = pb; B.slot_base[w] = sb;
        B.n_w[w] = lw.n; B.nid_w[w] = wi * D;
        B.max_n = std::max(B.max_n, lw.n);
        B.s_off[w] = so; B.simg_off[w] = sio; B.linv_off[w] = lo;
        so += (long long)lw.n * lw.n;
        sio += (long long)wi * D * wi * D;
        lo += (long long)div_up(lw.n, kCholNB) * kCholNB * kCholNB;
        for (int i = 0; i < wi; ++i) {
            B.cam_of_img.push_back(coi[i] + cb);
            L.pose_slot.push_back(lw.pose_slot[i] >= 0 ? lw.pose_slot[i] + sb : -1);
            L.img_active.push_back(lw.img_active[i]);
            L.img_free.push_back(lw.img_free[i]);
            B.img_win.push_back(w);
            for (int r = 0; r < D; ++r) {
                const int sl = lw.img_slot[(size_t)i * D + r];
                L.img_slot.push_back(sl >= 0 ? sl + sb : -1);
            }
        }
        for (int c = 0; c < wc; ++c) {
            B.model.push_back(mod[c]);
            L.cam_slot.push_back(lw.cam_slot[c] >= 0 ? lw.cam_slot[c] + sb : -1);
            B.cam_win.push_back(w);
        }
        const int pre_base = L.slot_pre_start.empty() ? 0 : L.slot_pre_start.back();
        if (L.slot_pre_start.empty()) L.slot_pre_start.push_back(0);
        for (int a = 0; a < lw.n; ++a) {
            L.slot_pre_start.push_back(pre_base + lw.slot_pre_start[a + 1]);
            L.slot_masked.push_back(lw.slot_masked[a]);
            B.slot_win.push_back(w);
        }
        for (int v : lw.slot_pre) L.slot_pre.push_back(v + ib * D);
        // Factorisation order: each image's pose slots, then its camera's
        // slots at the camera's first image, then any unreferenced camera.
        {
            std::vector<char> placed(lw.n, 0), cam_done(wc, 0);
            auto place = [&](int first, int count) {
                for (int k = 0; k < count; ++k)
                    if (!placed[first + k]) { placed[first + k] = 1; B.slot_perm.push_back(sb + first + k); }
            };
            for (int i = 0; i < wi; ++i) {
                if (lw.pose_slot[i] >= 0) place(lw.pose_slot[i], 6);
                const int c = coi[i];
                if (lw.cam_slot[c] >= 0 && !cam_done[c]) {
                    cam_done[c] = 1;
                    place(lw.cam_slot[c], model_dof(mod[c]));
                }
            }
            for (int a = 0; a < lw.n; ++a)
                if (!placed[a]) { placed[a] = 1; B.slot_perm.push_back(sb + a); }
        }
        B.cams.insert(B.cams.end(), p.camera_params, p.camera_params + (size_t)wc * 8);
        B.poses.insert(B.poses.end(), p.poses, p.poses + (size_t)wi * 7);
        B.fixed_pose.insert(B.fixed_pose.end(), fp.begin(), fp.end());
        B.fixed_cam.insert(B.fixed_cam.end(), fc.begin(), fc.end());
        B.fixed_cp.insert(B.fixed_cp.end(), fcp.begin(), fcp.end());
        {
            const int rows = std::max(1, 8192 / std::max(lw.n, 1));
            for (int r0 = 0; r0 < lw.n; r0 += rows) B.fold_blk.push_back(make_int4(w, r0, std::min(lw.n, r0 + rows), 0));
        }
        B.wblk_start.push_back((int)B.cblk_win.size());
        for (long long lo = ob; lo < ob + wo; lo += kWinCostChunk) {
            B.cblk_win.push_back(w);
            B.cblk_lo.push_back(lo);
        }
        ib += wi; cb += wc; pb += wp; sb += lw.n; ob += wo;
        B.obs_off[w + 1] = ob;
    }
    if (L.slot_pre_start.empty()) L.slot_pre_start.push_back(0);
    B.wblk_start.push_back((int)B.cblk_win.size());
    B.cblk_lo.push_back(ob);
    // Points and observations (the bulk of the batch), window by window on
    // the host threads into their final places.
    B.points.resize((size_t)nP * 3);
    B.win_of_point.resize(nP);
    B.obs_image.resize(nO);
    B.obs_point.resize(nO);
    B.obs_xy.resize((size_t)nO * 2);
    parallel_for(W, [&](int w) {
        const sfmba_problem &p = win[w];
        const long long o0 = B.obs_off[w];
        const int ib0 = B.img_base[w], pb0 = B.pt_base[w];
        std::copy(p.points, p.points + (size_t)p.num_points * 3, B.points.begin() + (size_t)pb0 * 3);
        std::fill(B.win_of_point.begin() + pb0, B.win_of_point.begin() + pb0 + p.num_points, w);
        for (long long o = 0; o < p.num_observations; ++o) {
            B.obs_image[o0 + o] = p.obs_image[o] + ib0;
            B.obs_point[o0 + o] = p.obs_point[o] + pb0;
        }
        std::copy(p.obs_xy, p.obs_xy + (size_t)p.num_observations * 2, B.obs_xy.begin() + (size_t)o0 * 2);
    });
    L.n = sb;
    B.s_total = so; B.simg_total = sio; B.linv_total = lo;
    sfmba_problem &q = B.problem;
    q.num_images = nI; q.num_cameras = nC; q.num_points = nP; q.num_observations = nO;
    q.camera_of_image = B.cam_of_img.data();
    q.camera_model = B.model.data();
    q.camera_params = B.cams.data();
    q.poses = B.poses.data();
    q.points = B.points.data();
    q.obs_image = B.obs_image.data();
    q.obs_point = B.obs_point.data();
    q.obs_xy = B.obs_xy.data();
    q.fixed_poses = B.fixed_pose.data();
    q.fixed_cameras = B.fixed_cam.data();
    q.fixed_camera_params = B.fixed_cp.data();
}

void check_options(const sfmba_options *o) {
    if (!o) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "options is NULL");
    if (o->max_iterations < 0) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "max_iterations < 0");
    if (o->robust_loss < 0 || o->robust_loss > 2) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "unknown robust_loss");
    if (o->precision < 0 || o->precision > 1) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "unknown precision");
    if (o->solver < 0 || o->solver > 2) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "unknown solver");
    if (!(o->initial_lambda >= 0.0) || !std::isfinite(o->initial_lambda))
        throw Error(SFMBA_ERR_INVALID_ARGUMENT, "initial_lambda must be finite and >= 0");
}

void check_problem_shape(const sfmba_problem *p) {
    if (!p) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "problem is NULL");
    if (p->num_images < 0 || p->num_cameras < 0 || p->num_points < 0 || p->num_observations < 0)
        throw Error(SFMBA_ERR_INVALID_ARGUMENT, "negative size");
    if (p->num_images > (1 << 20) || p->num_cameras > (1 << 20) || p->num_points > (1LL << 30) ||
        p->num_observations > (1LL << 31) - 1)
        throw Error(SFMBA_ERR_INVALID_ARGUMENT, "problem too large for 32-bit indices");
    auto need = [](const void *ptr, long long count, const char *name) {
        if (count > 0 && !ptr) throw Error(SFMBA_ERR_INVALID_ARGUMENT, std::string(name) + " is NULL");
    };
    need(p->camera_of_image, p->num_images, "camera_of_image");
    need(p->poses, p->num_images, "poses");
    need(p->camera_model, p->num_cameras, "camera_model");
    need(p->camera_params, p->num_cameras, "camera_params");
    need(p->points, p->num_points, "points");
    need(p->obs_image, p->num_observations, "obs_image");
    need(p->obs_point, p->num_observations, "obs_point");
    need(p->obs_xy, p->num_observations, "obs_xy");
}

void check_problem_host(const sfmba_problem *p) {
    for (long long c = 0; c < p->num_cameras; ++c)
        if (model_dof(p->camera_model[c]) == 0)
            throw Error(SFMBA_ERR_INVALID_ARGUMENT, "camera " + std::to_string(c) + " has an unknown model id");
    for (long long i = 0; i < p->num_images; ++i)
        if (p->camera_of_image[i] < 0 || p->camera_of_image[i] >= p->num_cameras)
            throw Error(SFMBA_ERR_INVALID_ARGUMENT, "camera_of_image[" + std::to_string(i) + "] out of range");
    // Observation indices: a branchless pass (16 host threads over fixed
    // chunks from 1M observations on); the first bad index is located only
    // to word the error.
    const long long nO = p->num_observations;
    const unsigned nI = (unsigned)p->num_images, nP = (unsigned)p->num_points;
    auto chunk_bad = [&](long long a, long long e) {
        unsigned bad = 0;
        for (long long o = a; o < e; ++o)
            bad |= (unsigned)((unsigned)p->obs_image[o] >= nI) | (unsigned)((unsigned)p->obs_point[o] >= nP);
        return bad != 0;
    };
    bool bad = false;
    const int nchunks = nO >= (1LL << 20) ? 16 : 1;
    if (nchunks > 1) {
        std::vector<char> flags(nchunks, 0);
        parallel_for(nchunks, [&](int k) { flags[k] = chunk_bad(nO * k / nchunks, nO * (k + 1) / nchunks); });
        for (char f : flags) bad = bad || f != 0;
    } else {
        bad = chunk_bad(0, nO);
    }
    if (!bad) return;
    for (long long o = 0; o < nO; ++o) {
        if (p->obs_image[o] < 0 || p->obs_image[o] >= p->num_images)
            throw Error(SFMBA_ERR_INVALID_ARGUMENT, "obs_image[" + std::to_string(o) + "] out of range");
        if (p->obs_point[o] < 0 || p->obs_point[o] >= p->num_points)
            throw Error(SFMBA_ERR_INVALID_ARGUMENT, "obs_point[" + std::to_string(o) + "] out of range");
    }
}

template <typename T>
std::vector<T> fetch(const T *src, size_t count, bool device, cudaStream_t s) {
    std::vector<T> v(count);
    if (count == 0) return v;
    if (device) {
        SFMBA_CUDA(cudaMemcpyAsync(v.data(), src, sizeof(T) * count, cudaMemcpyDeviceToHost, s));
        SFMBA_CUDA(cudaStreamSynchronize(s));
    } else {
        std::memcpy(v.data(), src, sizeof(T) * count);
    }
    return v;
}

template <typename T>
void put(T *dst, const T *src, size_t count, bool src_device, cudaStream_t s) {
    if (count == 0) return;
    SFMBA_CUDA(cudaMemcpyAsync(dst, src, sizeof(T) * count,
                               src_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
}

template <typename T>
void put_vec(T *dst, const std::vector<T> &v, cudaStream_t s) {
    if (v.empty()) return;
    SFMBA_CUDA(cudaMemcpyAsync(dst, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, s));
}

struct SolveOutput {
    double initial_cost = 0, final_cost = 0;
    int iterations = 0, retries = 0, solver = SFMBA_SOLVER_DENSE, polish_iteration = -1;
    long long linear_iterations = 0, valid_obs = 0;
    int n = 0;
};

class Solver {
  public:
    Solver(Context &ctx, cudaStream_t s) : ctx_(ctx), s_(s) {}

    // Clusters of consecutive images and the point-cluster pair groups of
    // the coarse correction (k_coarse.cu), once per solve. requested: 0 ->
    // kDefaultCoarseClusters, < 0 -> off.
    void setup_coarse(int requested) {
        Bufs &b = b_;
        CoarseBufs &co = b.co;
        co = CoarseBufs{};
        if (requested < 0 || b.nI < 2 || b.n == 0 || b.nP == 0) return;
        int nc = requested == 0 ? kDefaultCoarseClusters : std::min(requested, kMaxCoarseClusters);
        // At least kMinImagesPerCluster images per cluster: with one image per
        // cluster the coarse space repeats the block-Jacobi blocks and A_c is
        // the whole reduced system, whose FP32 inverse an ill-conditioned
        // problem does not survive; a few small clusters keep the smooth modes.
        nc = std::min(nc, b.nI / kMinImagesPerCluster);
        if (nc < 2) return;
        const int D = b.D, Nc = nc * D, nI = b.nI, nP = b.nP;
        std::vector<int> clu_start(nc + 1), img_cluster(nI);
        for (int c = 0; c <= nc; ++c) clu_start[c] = (int)((long long)c * nI / nc);
        for (int c = 0; c < nc; ++c)
            for (int i = clu_start[c]; i < clu_start[c + 1]; ++i) img_cluster[i] = c;
        Arena &A = ctx_.coarse;
        long long *count = nullptr, *off = nullptr, *kcount = nullptr;
        int *key_counts = nullptr;
        void *temp1 = nullptr;
        const size_t t1 = coarse_setup_temp_bytes(nP + 1, 1);
        for (int pass = 0; pass < 2; ++pass) {
            if (pass == 0) A.begin_sizing(); else A.commit();
            co.img_cluster = A.take<int>(nI);
            co.clu_start = A.take<int>((size_t)nc + 1);
            co.A = A.take<double>((size_t)Nc * Nc);
            co.X32 = A.take<float>((size_t)(2 * coarse_padded_size(Nc) + 2) * coarse_padded_size(Nc));
            co.fail = A.take<int>(2);
            co.Ainv = A.take<float>((size_t)Nc * Nc);
            co.cc = A.take<double>(Nc);
            co.zc = A.take<double>(Nc);
            co.zpart = A.take<double>((size_t)(div_up(nI, 8) + 1) * 3 * D);
            count = A.take<long long>((size_t)nP + 1);
            off = A.take<long long>((size_t)nP + 1);
            kcount = A.take<long long>((size_t)nP + 1);
            co.inc_off = A.take<long long>((size_t)nP + 1);
            key_counts = A.take<int>((size_t)nc * nc);
            temp1 = A.take<char>(t1);
        }
        put_vec(co.img_cluster, img_cluster, s_);
        put_vec(co.clu_start, clu_start, s_);
        SFMBA_CUDA(cudaMemsetAsync(kcount + nP, 0, sizeof(long long), s_));
        long long ninc = 0;
        const long long npairs = launch_coarse_count(b, count, off, kcount, co.inc_off, &ninc, temp1, t1, s_);
        if (npairs <= 0 || npairs > (1LL << 31) - 1 || ninc <= 0) {
            co = CoarseBufs{};
            return;
        }
        const int max_groups = nc * (nc + 1) / 2;
        const long long max_chunks = npairs / kCoarseChunk + max_groups + 1;
        Arena &P = ctx_.pairs;
        const size_t t2 = coarse_setup_temp_bytes(nP, npairs);
        int *key = nullptr, *val = nullptr, *key2 = nullptr, *val_sorted = nullptr;
        void *temp2 = nullptr;
        for (int pass = 0; pass < 2; ++pass) {
            if (pass == 0) P.begin_sizing(); else P.commit();
            key = P.take<int>(npairs);
            val = P.take<int>(npairs);
            key2 = P.take<int>(npairs);
            val_sorted = P.take<int>(npairs);
            temp2 = P.take<char>(t2);
            co.group_cc = P.take<int2>(max_groups);
            co.group_chunk_off = P.take<int>((size_t)max_groups + 1);
            co.chunk = P.take<int4>(max_chunks);
            co.chunk_part = P.take<double>((size_t)max_chunks * D * D);
            co.inc_cl = P.take<int>(ninc);
            co.inc_order = P.take<int>(ninc);
            co.inc_pt = P.take<int>(ninc);
            co.ybuf = P.take<double>((size_t)ninc * 3 * D);  // FP64-sized: an FP64 polish reuses it
        }
        co.ninc = ninc;
        co.nc = nc;
        launch_coarse_group(b, off, npairs, key, val, key2, val_sorted, key_counts, temp2, t2, s_);
        launch_coarse_inc_order(b, key, val, key2, temp2, t2, s_);  // the pair keys are consumed
        const std::vector<int> kc = fetch(key_counts, (size_t)nc * nc, true, s_);
        std::vector<int2> gcc;
        std::vector<int> goff{0};
        std::vector<int4> chunks;
        long long pos = 0;
        for (int k = 0; k < nc * nc; ++k) {
            const int cnt = kc[k];
            if (cnt == 0) continue;
            const int g = (int)gcc.size();
            gcc.push_back(make_int2(k / nc, k % nc));
            for (int a = 0; a < cnt; a += kCoarseChunk)
                chunks.push_back(make_int4(g, (int)(pos + a), (int)(pos + std::min(cnt, a + kCoarseChunk)), 0));
            goff.push_back((int)chunks.size());
            pos += cnt;
        }
        co.pair_pt = val_sorted;
        co.ngroups = (int)gcc.size();
        co.nchunks = (int)chunks.size();
        put_vec(co.group_cc, gcc, s_);
        put_vec(co.group_chunk_off, goff, s_);
        put_vec(co.chunk, chunks, s_);
    }

    // Shared free cameras on the PCG solver (k_shared.cu), once per solve:
    // the images of each shared camera, the (point, camera) incidences
    // sorted by camera and cut into chunks of kSharedChunk, and the buffers
    // of the per-retry camera blocks. tsz: element size of the kernel
    // precision (double when an FP64 polish may follow).
    void setup_shared(size_t tsz) {
        Bufs &b = b_;
        SharedBufs &sh = b.sh;
        const int nsh = (int)lay_.sh_img_start.size() - 1;
        const int nI = b.nI, nP = b.nP, D = b.D;
        const int KC = D - 6, NS = KC * (KC + 1) / 2;
        Arena &A = ctx_.shared;
        long long *count = nullptr;
        void *temp = nullptr;
        int *cam_counts = nullptr;
        size_t t1 = shared_setup_temp_bytes(nP, 1);
        for (int pass = 0; pass < 2; ++pass) {
            if (pass == 0) A.begin_sizing(); else A.commit();
            sh.img_owner = A.take<int>(nI);
            sh.img_shcam = A.take<int>(nI);
            sh.sh_img_start = A.take<int>((size_t)nsh + 1);
            sh.sh_imgs = A.take<int>(lay_.sh_imgs.size());
            sh.inc_off = A.take<long long>((size_t)nP + 1);
            sh.cam_chunk_off = A.take<int>((size_t)nsh + 1);
            cam_counts = A.take<int>(nsh);
            count = A.take<long long>((size_t)nP + 1);
            temp = A.take<char>(t1);
        }
        sh.nsh = nsh;
        put_vec(sh.img_owner, lay_.img_owner, s_);
        put_vec(sh.img_shcam, lay_.img_shcam, s_);
        put_vec(sh.sh_img_start, lay_.sh_img_start, s_);
        put_vec(sh.sh_imgs, lay_.sh_imgs, s_);
        sh.ninc = launch_shared_count(b, count, temp, t1, s_);
        if (sh.ninc > (1LL << 31) - 1)
            throw Error(SFMBA_ERR_UNSUPPORTED, "too many point-camera incidences for the shared-camera blocks");
        const size_t t2 = shared_setup_temp_bytes(nP, sh.ninc);
        Arena &P = ctx_.shared_inc;
        int *key = nullptr, *val = nullptr, *key2 = nullptr;
        void *temp2 = nullptr;
        const long long max_chunks = sh.ninc / kSharedChunk + nsh + 1;
        for (int pass = 0; pass < 2; ++pass) {
            if (pass == 0) P.begin_sizing(); else P.commit();
            key = P.take<int>(sh.ninc);
            val = P.take<int>(sh.ninc);
            key2 = P.take<int>(sh.ninc);
            temp2 = P.take<char>(t2);
            sh.inc_sorted = P.take<int>(sh.ninc);
            sh.inc_W = P.take<char>((size_t)sh.ninc * NS * tsz);
            sh.chunk = P.take<int4>(max_chunks);
            sh.chunk_part = P.take<double>((size_t)max_chunks * NS);
        }
        launch_shared_sort(b, key, val, key2, cam_counts, temp2, t2, s_);
        const std::vector<int> cnt = fetch(cam_counts, (size_t)nsh, true, s_);
        std::vector<int4> chunks;
        std::vector<int> off{0};
        int pos = 0;
        for (int c = 0; c < nsh; ++c) {
            for (int a = 0; a < cnt[c]; a += kSharedChunk)
                chunks.push_back(make_int4(c, pos + a, pos + std::min(cnt[c], a + kSharedChunk), 0));
            off.push_back((int)chunks.size());
            pos += cnt[c];
        }
        sh.nchunks = (int)chunks.size();
        put_vec(sh.chunk, chunks, s_);
        put_vec(sh.cam_chunk_off, off, s_);
        SFMBA_CUDA(cudaStreamSynchronize(s_));  // host vectors above go out of scope
    }

    // A_c for this retry and its FP32 inverse; false (block-Jacobi alone
    // for this retry) when the sweep breaks down.
    bool factor_coarse() {
        Bufs &b = b_;
        CoarseBufs &co = b.co;
        if (co.nc == 0) return false;
        { SFMBA_PHASE(PH_COARSE_ASSEMBLE); launch_coarse_assemble(b, s_); }
        SFMBA_PHASE(PH_COARSE_FACTOR);
        launch_coarse_invert(b, s_);
        int st[2] = {1, 0};
        SFMBA_CUDA(cudaMemcpyAsync(st, co.fail, sizeof(st), cudaMemcpyDeviceToHost, s_));
        SFMBA_CUDA(cudaStreamSynchronize(s_));
        profiler().count("coarse_inverses", 1);
        profiler().count("coarse_inverse_failed", st[0]);
        profiler().count("coarse_pivots_raised", st[1]);
        return st[0] == 0;
    }

    void read_state() {
        SFMBA_CUDA(cudaMemcpyAsync(ctx_.h_state, b_.state, sizeof(LMState), cudaMemcpyDeviceToHost, s_));
        SFMBA_CUDA(cudaStreamSynchronize(s_));
    }

    // Copies the problem into solver layout and builds all device structures.
    void setup(const sfmba_problem *p, const sfmba_options *o, bool device, bool need_system,
               const Batch *batch = nullptr) {
        const int nI = (int)p->num_images, nC = (int)p->num_cameras, nP = (int)p->num_points;
        const long long nO = p->num_observations;
        StageClock clk(s_);
        std::vector<int> cam_of_img = fetch(p->camera_of_image, nI, device, s_);
        std::vector<int> model = fetch(p->camera_model, nC, device, s_);
        for (int c = 0; c < nC; ++c)
            if (model_dof(model[c]) == 0)
                throw Error(SFMBA_ERR_INVALID_ARGUMENT, "camera " + std::to_string(c) + " has an unknown model id");
        for (int i = 0; i < nI; ++i)
            if (cam_of_img[i] < 0 || cam_of_img[i] >= nC)
                throw Error(SFMBA_ERR_INVALID_ARGUMENT, "camera_of_image[" + std::to_string(i) + "] out of range");
        std::vector<unsigned char> fp(nI, 0), fc(nC, 0), fcp((size_t)nC * 8, 0);
        if (p->fixed_poses) fp = fetch(p->fixed_poses, nI, device, s_);
        if (p->fixed_cameras) fc = fetch(p->fixed_cameras, nC, device, s_);
        if (p->fixed_camera_params) fcp = fetch(p->fixed_camera_params, (size_t)nC * 8, device, s_);
        lay_ = batch ? batch->lay : make_layout(nI, nC, nP, nO, cam_of_img, model, fp, fc, fcp);
        const int n = lay_.n, D = lay_.D;
        const bool mixed = o->precision == SFMBA_PRECISION_MIXED;
        solver_ = SFMBA_SOLVER_DENSE;
        if (batch) {
            // every window is solved densely; its own size limit was checked
        } else if (o->solver == SFMBA_SOLVER_PCG) solver_ = SFMBA_SOLVER_PCG;
        else if (o->solver == SFMBA_SOLVER_AUTO)
            solver_ = (n <= std::max(1, o->dense_max_dim)) ? SFMBA_SOLVER_DENSE : SFMBA_SOLVER_PCG;
        // The dense path holds S, its factor and the image-level Schur blocks
        // (3 n^2 + (nI D)^2 doubles); larger systems go to the PCG solver,
        // which takes every camera-sharing pattern (k_shared.cu).
        if (!batch && solver_ == SFMBA_SOLVER_DENSE && (n > kDenseMaxDim || nI > 65535)) solver_ = SFMBA_SOLVER_PCG;
        const int nID = nI * D;
        // The mixed path may finish in FP64 (fp64_polish): its typed buffers
        // are sized for doubles so the same allocation serves both precisions.
        const bool polish = mixed && o->fp64_polish;
        const size_t tsz = (mixed && !polish) ? sizeof(float) : sizeof(double);
        const size_t RS = (size_t)((8 + 2 * D) + 3) / 4 * 4;
        size_t sort_tmp = sort_temp_bytes(std::max<long long>(nO, 1), std::max(nP, 1), nI);
        {
            size_t scan_bytes = 0;
            SFMBA_CUDA(cub::DeviceScan::InclusiveSum(nullptr, scan_bytes, (long long *)nullptr,
                                                     (long long *)nullptr, std::max(nP, 1)));
            sort_tmp = std::max(sort_tmp, scan_bytes);
        }

        Arena &A = ctx_.main;
        int *in_img = nullptr, *in_pt = nullptr;
        double *in_xy = nullptr;
        void *sort_temp = nullptr;
        int *k1 = nullptr, *v1 = nullptr, *k2 = nullptr, *v2 = nullptr;
        long long *pair_scan = nullptr;
        int *d_bad = nullptr;
        int *pkey = nullptr, *pkey2 = nullptr, *piota = nullptr, *obs_pt_new = nullptr;
        int *win_in = nullptr;
        for (int pass = 0; pass < 2; ++pass) {
            if (pass == 0) A.begin_sizing(); else A.commit();
            Bufs &b = b_;
            b = Bufs();
            w_ = WinBufs();
            if (batch) {
                const int W = batch->W;
                w_.W = W;
                w_.max_n = batch->max_n;
                w_.ws = A.take<WinState>(W);
                w_.pt_win = A.take<int>(nP);
                w_.img_win = A.take<int>(nI);
                w_.cam_win = A.take<int>(nC);
                w_.slot_win = A.take<int>(n);
                w_.img_base = A.take<int>(W);
                w_.nid_w = A.take<int>(W);
                w_.n_w = A.take<int>(W);
                w_.slot_base = A.take<int>(W);
                w_.s_off = A.take<long long>(W);
                w_.simg_off = A.take<long long>(W);
                w_.linv_off = A.take<long long>(W);
                w_.obs_off = A.take<long long>((size_t)W + 1);
                w_.counts = A.take<int>(4);
                w_.slot_perm = A.take<int>(n);
                const int ncb = (int)batch->cblk_win.size();
                w_.ncblk = ncb;
                w_.cblk_win = A.take<int>(ncb);
                w_.cblk_lo = A.take<long long>((size_t)ncb + 1);
                w_.wblk_start = A.take<int>((size_t)W + 1);
                w_.cpart = A.take<double>(ncb);
                w_.cpart_n = A.take<long long>(ncb);
                w_.row_first = A.take<int>(n);
                w_.rhs_p = A.take<double>(n);
                w_.lu_list = A.take<int>(W);
                w_.n_fold_blk = (int)batch->fold_blk.size();
                w_.fold_blk = A.take<int4>(batch->fold_blk.size());
                w_.lu_count = A.take<int>(1);
                win_in = A.take<int>(nP);
                b.img_live = A.take<unsigned char>(nI);
                b.pt_live = A.take<unsigned char>(nP);
            }
            b.nI = nI; b.nC = nC; b.nP = nP; b.nO = nO; b.n = n; b.D = D; b.nID = nID;
            b.mixed = mixed; b.loss = o->robust_loss; b.loss_scale = o->loss_scale_px;
            b.uniform_model = nC > 0 ? model[0] : -1;
            for (int c = 1; c < nC; ++c)
                if (model[c] != b.uniform_model) { b.uniform_model = -1; break; }
            b.pcg_tol = o->pcg_tolerance > 0.0 ? o->pcg_tolerance : 0.1;
            b.cam_model = A.take<int>(nC);
            b.cam_of_img = A.take<int>(nI);
            b.cams = A.take<double>((size_t)nC * 8);
            b.cams_trial = A.take<double>((size_t)nC * 8);
            b.poses = A.take<double>((size_t)nI * 7);
            b.poses_trial = A.take<double>((size_t)nI * 7);
            b.points = A.take<double>((size_t)nP * 3);
            b.points_trial = A.take<double>((size_t)nP * 3);
            b.points32 = mixed ? A.take<float4>(nP) : nullptr;
            b.ob_img = A.take<int>(nO);
            b.ob_pt = A.take<int>(nO);
            b.ob_xy = A.take<double2>(nO);
            b.pt_start = A.take<int>((size_t)nP + 1);
            b.img_start = A.take<int>((size_t)nI + 1);
            b.img_obs = A.take<int>(nO);
            b.img_slot = A.take<int>((size_t)nID);
            b.img_active = A.take<int>(nI);
            b.img_pmask = A.take<int>(nI);
            b.img_dmask = A.take<int>(nI);
            b.img_free = A.take<int>(nI);
            b.cam_slot = A.take<int>(nC);
            b.pose_slot = A.take<int>(nI);
            b.slot_pre_start = A.take<int>((size_t)n + 1);
            b.slot_pre = A.take<int>(lay_.slot_pre.size());
            b.slot_masked = A.take<unsigned char>(n);
            b.state = A.take<LMState>(1);
            b.partials = A.take<double>(kCostBlocks);
            b.img_rt64 = A.take<double>((size_t)nI * 12 + 1);
            // Double-float cost buffers: FP32 path, no fisheye camera.
            bool df = mixed;
            for (int c = 0; c < nC && df; ++c) df = model[c] != SFMBA_OPENCV_FISHEYE;
            b.df_cost = df ? 1 : 0;
            b.ob_xy_df = df ? A.take<float4>(nO) : nullptr;
            b.pts_df = df ? A.take<float4>((size_t)nP * 2) : nullptr;
            b.rt_df = df ? A.take<float>((size_t)nI * 24 + 4) : nullptr;
            b.cams_df = df ? A.take<float>((size_t)nC * 16 + 4) : nullptr;
            b.count_partials = A.take<long long>(kCostBlocks);
            d_bad = A.take<int>(1);
            if (!device) {
                in_img = A.take<int>(nO);
                in_pt = A.take<int>(nO);
                in_xy = A.take<double>((size_t)nO * 2);
            }
            if (need_system) {
                const bool records = solver_ == SFMBA_SOLVER_DENSE || !mixed || polish;
                const long long nchunks = (nO + kChunkObs - 1) / kChunkObs;
                b.img_lin = A.take<char>((size_t)nI * sizeof(ImageLin<double>));
                b.ob_rs = mixed ? A.take<float4>(nO) : nullptr;
                b.ob_rs_trial = mixed ? A.take<float4>(nO) : nullptr;
                b.rec = records ? A.take<char>((size_t)nO * RS * tsz) : nullptr;
                b.ob_valid = A.take<unsigned char>(nO);
                b.pt_C = A.take<char>((size_t)nP * 6 * tsz);
                b.pt_g = A.take<char>((size_t)nP * 3 * tsz);
                b.pt_nfree = A.take<int>(nP);
                b.pt_Cinv = A.take<char>((size_t)nP * 6 * tsz);
                b.pt_h = A.take<char>((size_t)nP * 3 * tsz);
                b.pt_ok = A.take<unsigned char>(nP);
                b.img_H = A.take<double>((size_t)nID * D);
                b.img_b = A.take<double>((size_t)nID);
                b.img_rhs = A.take<double>((size_t)nID);
                b.img_delta = A.take<char>((size_t)nID * tsz);
                // Image-aligned chunks, their partials and the image-major packed
                // records of the image-block passes (H_i, b_i; PCG preconditioner).
                b.ipart2 = A.take<char>((size_t)(nI + nchunks + 1) * 2 * (D * (D + 1) / 2 + D) * tsz);  // fused: 2 sums
                b.iachunk = A.take<int4>((size_t)(nI + nchunks + 1));
                b.iachunk_off = A.take<int>((size_t)nI + 1);
                b.isrec = A.take<int4>(nO);
                b.rhs = A.take<double>(n);
                b.delta = A.take<double>(n);
                b.diagB = A.take<double>(n);
                b.work = A.take<double>(n);
                b.work2 = A.take<double>(n);
                b.ref_res = A.take<double>(n);
                b.ref_corr = A.take<double>(n);
                if (batch) {
                    b.S_img = A.take<double>((size_t)batch->simg_total);
                    b.S = A.take<double>((size_t)batch->s_total);
                    b.L = A.take<double>((size_t)batch->s_total);
                    b.Linv = A.take<double>((size_t)batch->linv_total);
                    b.lu_perm = A.take<int>(n);
                    pair_scan = A.take<long long>(nP);
                    b.oz_slices = nullptr;
                    b.oz_exp = nullptr;
                    if (mixed && !o->dense_fp64_fma) {  // tensor-core trailing updates (ozaki.cuh)
                        b.oz_slices = A.take<uint16_t>((size_t)kOzSlices * n * kOzK);
                        b.oz_exp = A.take<int>(n);
                    }
                } else if (solver_ == SFMBA_SOLVER_DENSE) {
                    b.S_img = A.take<double>((size_t)nID * nID);
                    b.S = A.take<double>((size_t)n * n);
                    b.L = A.take<double>((size_t)n * n);
                    b.Linv = A.take<double>((size_t)div_up(n, kCholNB) * kCholNB * kCholNB);
                    b.lu_perm = A.take<int>(n);
                    pair_scan = A.take<long long>(nP);
                    b.oz_slices = nullptr;
                    b.oz_exp = nullptr;
                    if (mixed && !o->dense_fp64_fma) {  // tensor-core trailing updates (ozaki.cuh)
                        b.oz_slices = A.take<uint16_t>((size_t)2 * kOzSlices * n * kOzK);
                        b.oz_exp = A.take<int>((size_t)2 * n);
                    }
                } else {
                    b.pcg_x = A.take<char>((size_t)nID * tsz);
                    b.pcg_r = A.take<char>((size_t)nID * tsz);
                    b.pcg_z = A.take<char>((size_t)nID * tsz);
                    b.pcg_p = A.take<char>((size_t)nID * tsz);
                    b.pcg_p4 = mixed ? A.take<float>((size_t)nI * pad4(D)) : nullptr;
                    b.img_mv = mixed ? A.take<float4>((size_t)5 * nI) : nullptr;
                    b.pcg_q = A.take<char>((size_t)nID * tsz);
                    b.pcg_u = A.take<char>((size_t)nP * 4 * tsz);
                    b.pcg_Minv = A.take<char>((size_t)nID * D * tsz);
                    b.img_Hf = mixed ? A.take<float>((size_t)nID * D) : nullptr;
                    b.pcg_part = A.take<double>((size_t)3 * nI);  // r.z, r.r, p.q per image
                    b.pcg_blk = A.take<double>((size_t)4 * kPcgMaxCoopBlocks);
                    b.pchunk = A.take<int>((size_t)nchunks + 1);
                    b.ipart_off = A.take<int>((size_t)nI + 1);
                    b.ipart = A.take<char>((size_t)(nI + nchunks + 1) * D * tsz);
                    b.obrec = A.take<int4>(nO);
                }
            }
            if (need_system) {
                b.pt_perm = A.take<int>(nP);
                b.pt_old2new = A.take<int>(nP);
                pkey = A.take<int>(nP);
                pkey2 = A.take<int>(nP);
                piota = A.take<int>(nP);
                obs_pt_new = A.take<int>(nO);
            }
            sort_temp = A.take<char>(sort_tmp);
            k1 = A.take<int>(nO);
            v1 = A.take<int>(nO);
            k2 = A.take<int>(nO);
            v2 = A.take<int>(nO);
        }
        Bufs &b = b_;
        clk.mark("setup_layout");
        // Problem arrays.
        put(const_cast<int *>(b.cam_model), p->camera_model, nC, device, s_);
        put(const_cast<int *>(b.cam_of_img), p->camera_of_image, nI, device, s_);
        put(b.cams, p->camera_params, (size_t)nC * 8, device, s_);
        put(b.poses, p->poses, (size_t)nI * 7, device, s_);
        if (!need_system) put(b.points, p->points, (size_t)nP * 3, device, s_);
        const int *src_img = p->obs_image, *src_pt = p->obs_point;
        const double *src_xy = p->obs_xy;
        if (!device) {
            put(in_img, p->obs_image, nO, false, s_);
            put(in_pt, p->obs_point, nO, false, s_);
            put(in_xy, p->obs_xy, (size_t)nO * 2, false, s_);
            src_img = in_img; src_pt = in_pt; src_xy = in_xy;
        } else {
            SFMBA_CUDA(cudaMemsetAsync(d_bad, 0, sizeof(int), s_));
            validate_problem_device(b.cam_of_img, b.cam_model, src_img, src_pt, nO, nI, nC, nP, d_bad, s_);
            int bad = 0;
            SFMBA_CUDA(cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, s_));
            SFMBA_CUDA(cudaStreamSynchronize(s_));
            if (bad) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "observation, image or camera index out of range");
        }
        put_vec(b.img_slot, lay_.img_slot, s_);
        put_vec(b.img_active, lay_.img_active, s_);
        put_vec(b.img_pmask, lay_.img_pmask, s_);
        put_vec(b.img_dmask, lay_.img_dmask, s_);
        put_vec(b.img_free, lay_.img_free, s_);
        put_vec(b.cam_slot, lay_.cam_slot, s_);
        put_vec(b.pose_slot, lay_.pose_slot, s_);
        put_vec(b.slot_pre_start, lay_.slot_pre_start, s_);
        put_vec(b.slot_pre, lay_.slot_pre, s_);
        put_vec(b.slot_masked, lay_.slot_masked, s_);
        clk.mark("setup_upload");
        if (need_system) {
            // Solver point order: by first observing image (see order_points).
            order_points(src_pt, src_img, nO, nP, nI, pkey, pkey2, piota, b.pt_perm, b.pt_old2new, obs_pt_new,
                         sort_temp, sort_tmp, s_);
            put(b.points_trial, p->points, (size_t)nP * 3, device, s_);
            gather_points(b.points_trial, b.pt_perm, nP, b.points, s_);
            src_pt = obs_pt_new;
        }
        sort_observations(src_pt, src_img, src_xy, nO, nP, nI, b, sort_temp, sort_tmp, k1, v1, k2, v2, s_);
        launch_split_xy_df(b, s_);
        SFMBA_CUDA(cudaMemsetAsync(b.state, 0, sizeof(LMState), s_));
        clk.mark("setup_sort");
        if (need_system) {
            std::vector<int> img_start = fetch(b.img_start, (size_t)nI + 1, true, s_);
            if (solver_ == SFMBA_SOLVER_PCG) {
                launch_pcg_partition(b, s_);
                // Partial-sum slots of the image pass: one per (chunk, image) overlap.
                std::vector<int> off(nI + 1, 0);
                for (int i = 0; i < nI; ++i) {
                    const int a = img_start[i], e = img_start[i + 1];
                    off[i + 1] = off[i] + (e > a ? (e - 1) / kChunkObs - a / kChunkObs + 1 : 0);
                }
                b.nparts = off[nI];
                put_vec(b.ipart_off, off, s_);
                clk.mark("setup_partition");
                setup_coarse(o->pcg_coarse_clusters);
                clk.mark("setup_coarse");
                b.sh = SharedBufs();
                if (lay_.sh_img_start.size() > 1) setup_shared(tsz);
            }
            // Image-aligned chunks of the image-block passes.
            std::vector<int4> ia;
            std::vector<int> ia_off(nI + 1, 0);
            for (int i = 0; i < nI; ++i) {
                ia_off[i] = (int)ia.size();
                for (int lo = img_start[i]; lo < img_start[i + 1]; lo += kChunkObs)
                    ia.push_back(make_int4(i, lo, std::min(lo + kChunkObs, img_start[i + 1]), 0));
            }
            ia_off[nI] = (int)ia.size();
            b.n_iachunks = (int)ia.size();
            put_vec(b.iachunk, ia, s_);
            put_vec(b.iachunk_off, ia_off, s_);
            if (b.pcg_p4) SFMBA_CUDA(cudaMemsetAsync(b.pcg_p4, 0, sizeof(float) * (size_t)nI * pad4(D), s_));
            launch_mf_prepare(b, s_);
            clk.mark("setup_chunks");
        }
        if (need_system && solver_ == SFMBA_SOLVER_DENSE && n > 0) {
            // pair count scan uses the sort temp (cub scan needs little)
            b.npairs = count_pairs(b, pair_scan, sort_temp, sort_tmp, s_);
            if (b.npairs > (1LL << 31) - 1)
                throw Error(SFMBA_ERR_UNSUPPORTED, "too many observation pairs for the dense Schur path");
            const size_t ptemp = pairs_temp_bytes(b.npairs, nI);
            Arena &P = ctx_.pairs;
            unsigned *ka = nullptr, *kb = nullptr;
            int2 *vb = nullptr;
            void *pt = nullptr;
            int *d_ng = nullptr;
            for (int pass = 0; pass < 2; ++pass) {
                if (pass == 0) P.begin_sizing(); else P.commit();
                b.pairs = P.take<int2>(b.npairs);
                b.group_start = P.take<int>(b.npairs + 1);
                b.group_ij = P.take<int2>(b.npairs);
                b.group_order = P.take<int>(b.npairs);
                ka = P.take<unsigned>(b.npairs);
                kb = P.take<unsigned>(b.npairs);
                vb = P.take<int2>(b.npairs + 1);
                pt = P.take<char>(ptemp);
                d_ng = P.take<int>(1);
            }
            build_pairs(b, pair_scan, ka, kb, vb, pt, ptemp, d_ng, s_);
            const size_t simg = batch ? (size_t)batch->simg_total : (size_t)nID * nID;
            SFMBA_CUDA(cudaMemsetAsync(b.S_img, 0, sizeof(double) * simg, s_));
        }
        if (batch) {
            WinBufs &w = w_;
            put_vec(w.img_win, batch->img_win, s_);
            put_vec(w.cam_win, batch->cam_win, s_);
            put_vec(w.slot_win, batch->slot_win, s_);
            put_vec(w.img_base, batch->img_base, s_);
            put_vec(w.nid_w, batch->nid_w, s_);
            put_vec(w.n_w, batch->n_w, s_);
            put_vec(w.slot_base, batch->slot_base, s_);
            put_vec(w.s_off, batch->s_off, s_);
            put_vec(w.simg_off, batch->simg_off, s_);
            put_vec(w.linv_off, batch->linv_off, s_);
            put_vec(w.obs_off, batch->obs_off, s_);
            put_vec(w.slot_perm, batch->slot_perm, s_);
            put_vec(w.cblk_win, batch->cblk_win, s_);
            put_vec(w.fold_blk, batch->fold_blk, s_);
            put_vec(w.cblk_lo, batch->cblk_lo, s_);
            put_vec(w.wblk_start, batch->wblk_start, s_);
            put_vec(win_in, batch->win_of_point, s_);
            launch_wb_window_of_points(win_in, b.pt_perm, nP, w.pt_win, s_);
        }
        if (mixed) launch_refresh_points32(b, s_);
        clk.mark("setup_rest");
    }

    SolveOutput run(const sfmba_options *o) {
        SolveOutput out;
        Bufs &b = b_;
        out.n = b.n;
        out.solver = solver_;
        LMState &hs = *ctx_.h_state;
        // initial cost (lib.rs:794)
        { SFMBA_PHASE(PH_COST); launch_cost(b, false, false, s_); }
        {
            LMState init{};
            init.lambda = o->initial_lambda;
            init.nu = 2.0;
            // cost and valid_obs were just written by launch_cost; keep them
            read_state();
            init.cost = hs.cost;
            init.valid_obs = hs.valid_obs;
            SFMBA_CUDA(cudaMemcpyAsync(b.state, &init, sizeof(LMState), cudaMemcpyHostToDevice, s_));
            SFMBA_CUDA(cudaStreamSynchronize(s_));
            out.initial_cost = init.cost;
            out.final_cost = init.cost;
            out.valid_obs = init.valid_obs;
        }
        if (b.n == 0) return out;  // lib.rs:777-787
        bool polish_pending = b.mixed && o->fp64_polish;
        for (int outer = 0; outer < o->max_iterations; ++outer) {
            ++out.iterations;
            { SFMBA_PHASE(PH_LM); launch_begin_outer(b, s_); }
            {
                SFMBA_PHASE(PH_LINEARIZE);
                launch_prepare_images(b, s_);
                if (solver_ == SFMBA_SOLVER_DENSE || !b.mixed) launch_linearize(b, s_);
            }
            if (solver_ == SFMBA_SOLVER_DENSE) {
                { SFMBA_PHASE(PH_POINT_REDUCE); launch_point_reduce(b, s_); }
                { SFMBA_PHASE(PH_IMAGE_REDUCE); launch_image_blocks_records(b, s_); launch_diag_fold(b, s_); }
            } else {
                { SFMBA_PHASE(PH_POINT_REDUCE); launch_mf_point_reduce(b, s_); }
                // FP32: H_i and b_i come with the preconditioner's pass in each retry.
                if (!b.mixed) { SFMBA_PHASE(PH_IMAGE_REDUCE); launch_mf_image_blocks(b, s_); }
            }
            read_state();
            // lib.rs:855-857: no observation in front of its camera
            if (hs.valid_obs == 0) break;
            const double lambda_start = hs.lambda, nu_start = hs.nu;
            bool accepted = false;
            for (int inner = 0; inner < kMaxDampingRetries; ++inner) {
                ++out.retries;
                { SFMBA_PHASE(PH_LM); launch_begin_retry(b, s_); }
                { SFMBA_PHASE(PH_POINT_INVERSE); launch_point_inverse(b, s_); }
                if (solver_ == SFMBA_SOLVER_DENSE) {
                    { SFMBA_PHASE(PH_IMAGE_RHS); launch_image_rhs(b, s_); }
                    { SFMBA_PHASE(PH_SCHUR); launch_schur_pairs(b, s_); }
                    { SFMBA_PHASE(PH_FOLD); launch_fold_system(b, s_); }
                    { SFMBA_PHASE(PH_CHOLESKY); launch_cholesky(b, s_); }
                    { SFMBA_PHASE(PH_TRSV); launch_cholesky_solve(b, b.rhs, b.delta, s_); }
                    if (b.mixed) {
                        SFMBA_PHASE(PH_REFINE);
                        for (int k = 0; k < o->refinement_steps; ++k) launch_refine(b, s_);
                    }
                    { SFMBA_PHASE(PH_BACKSUB); launch_backsub_update(b, b.delta, s_); }
                } else {
                    const bool fused = b.mixed;  // H_i, b_i and the preconditioner in one pass
                    if (fused) { SFMBA_PHASE(PH_PCG_PRECOND); launch_mf_precond_fused(b, s_); }
                    bool coarse = false;
                    if (b.co.nc > 0) {  // the assembly reads H_i
                        // The coarse inverse is refreshed when the damping has moved by 100x
                        // or 6 outer iterations have passed since it was formed; in between
                        // the previous one (still symmetric positive definite) is used.
                        const double lam = hs.lambda;
                        if (!coarse_valid_ || outer - coarse_outer_ >= 6 || lam < coarse_lambda_ * 0.01 ||
                            lam > coarse_lambda_ * 100.0) {
                            coarse_valid_ = factor_coarse();
                            coarse_lambda_ = lam;
                            coarse_outer_ = outer;
                        }
                        coarse = coarse_valid_;
                    }
                    {
                        SFMBA_PHASE(PH_PCG_PRECOND);
                        if (!fused) launch_mf_precond(b, s_);
                        if (b.sh.nsh > 0) launch_shared_precond(b, s_);
                        if (coarse) launch_coarse_correct(b, true, s_);
                        launch_pcg_start(b, s_);
                    }
                    const int maxit = std::max(1, o->pcg_max_iterations);
                    int vp = 0, vi = 0;  // launch variants of the two passes
                    if (o->kernel_variant > 0) {
                        vp = std::min(o->kernel_variant, kPointPassVariants) - 1;
                        vi = (o->kernel_variant - 1) % kImagePassVariants;
                    } else if (b.mixed) {
                        vp = tuned_variant(ctx_.device, 0, kPointPassVariants, b, s_,
                                           [&](int v) { launch_mf_points(b, s_, v); });
                        vi = tuned_variant(ctx_.device, 1, kImagePassVariants, b, s_,
                                           [&](int v) { launch_mf_images(b, s_, v); });
                    }
                    // With the phase profiler on, convergence is polled after every
                    // iteration, so every profiled pass launch does an iteration's work
                    // (otherwise up to 7 launches per solve return at once).
                    const int poll = profiler().on ? 1 : kPcgPollEvery;
                    for (int it = 0; it < maxit; it += poll) {
                        const int m = std::min(poll, maxit - it);
                        auto chunk = [&] {
                            for (int k = 0; k < m; ++k) {
                                { SFMBA_PHASE(PH_PCG_POINTS); launch_mf_points(b, s_, vp); }
                                { SFMBA_PHASE(PH_PCG_IMAGES); launch_mf_images(b, s_, vi); }
                                { SFMBA_PHASE(PH_PCG_VECTOR); launch_pcg_iteration_vector(b, s_, (it + k) & 1, coarse); }
                            }
                        };
                        pcg_chunk_[coarse ? 1 : 0].run(s_, m == kPcgPollEvery && !profiler().on, chunk);
                        read_state();
                        if (hs.wait_timeouts)
                            throw Error(SFMBA_ERR_INTERNAL, "a bounded wait of the TMA point pass gave up");
                        if (hs.pcg_done) break;
                    }
                    { SFMBA_PHASE(PH_PCG_VECTOR); launch_pcg_finish(b, b.delta, s_); }
                    { SFMBA_PHASE(PH_BACKSUB); launch_mf_backsub(b, b.delta, s_); }
                }
                { SFMBA_PHASE(PH_COST); launch_cost(b, true, true, s_); }
                { SFMBA_PHASE(PH_LM); launch_accept(b, s_); launch_commit(b, s_); }
                read_state();
                if (hs.factor_failed) {
                    // LU fallback on the symmetrised system (lib.rs:1084-1092)
                    { SFMBA_PHASE(PH_LU); launch_lu_factor(b, s_); launch_lu_solve(b, s_); }
                    { SFMBA_PHASE(PH_BACKSUB); launch_backsub_update(b, b.delta, s_); }
                    { SFMBA_PHASE(PH_COST); launch_cost(b, true, true, s_); }
                    { SFMBA_PHASE(PH_LM); launch_accept(b, s_); launch_commit(b, s_); launch_reject(b, s_); }
                    read_state();
                }
                if (hs.accepted) {
                    accepted = true;
                    break;
                }
            }
            bool stop = !accepted;
            if (profiler().on) {
                char tmp[320];
                std::snprintf(tmp, sizeof(tmp),
                              "{\"outer\":%d,\"accepted\":%d,\"fp32\":%d,\"cost\":%.17g,\"cost_before\":%.17g,"
                              "\"lambda\":%.6g,\"retries\":%d,\"pcg_total\":%lld,\"pcg_breakdowns\":%d}",
                              outer, accepted ? 1 : 0, b.mixed, hs.cost, hs.cost_before, hs.lambda, out.retries,
                              hs.pcg_total, hs.pcg_breakdowns);
                profiler().trace.push_back(tmp);
            }
            if (accepted) {
                out.final_cost = hs.cost;
                out.valid_obs = hs.valid_obs;
                const double rel = (hs.cost_before - hs.cost) / std::max(hs.cost_before, 1e-12);
                if (o->target_cost > 0.0 && hs.cost <= o->target_cost) break;
                stop = rel < kFunctionTolerance;
            }
            if (!stop) continue;
            if (polish_pending && std::isfinite(hs.cost)) {
                // The FP32 loop would stop here (lib.rs:1215-1221 rules): continue the
                // same loop in FP64. A failed iteration's damping growth is undone.
                polish_pending = false;
                b.mixed = 0;
                for (auto &g : pcg_chunk_) g.reset();  // the captured FP32 chunks do not apply any more
                out.polish_iteration = outer + 1;
                if (!accepted) {
                    SFMBA_CUDA(cudaMemcpyAsync(&b.state->lambda, &lambda_start, sizeof(double),
                                               cudaMemcpyHostToDevice, s_));
                    SFMBA_CUDA(cudaMemcpyAsync(&b.state->nu, &nu_start, sizeof(double), cudaMemcpyHostToDevice, s_));
                    SFMBA_CUDA(cudaStreamSynchronize(s_));
                }
                continue;
            }
            break;
        }
        read_state();
        out.final_cost = hs.cost;
        out.valid_obs = hs.valid_obs;
        out.linear_iterations = hs.pcg_total;
        return out;
    }

    // The LM loop of every window of a batch (lib.rs:794-1232 per window).
    // Each kernel covers all windows; the windows that take part in a retry
    // are flagged on the device, and the host only reads four counts per
    // retry to decide whether another round is needed.
    std::vector<WinState> run_batched(const sfmba_options *o) {
        Bufs &b = b_;
        WinBufs &w = w_;
        int *hc = ctx_.h_counts;
        auto counts = [&] {
            launch_wb_summary(w, s_);
            SFMBA_CUDA(cudaMemcpyAsync(hc, w.counts, 4 * sizeof(int), cudaMemcpyDeviceToHost, s_));
            SFMBA_CUDA(cudaStreamSynchronize(s_));
        };
        { SFMBA_PHASE(PH_COST); launch_wb_cost(b, w, false, s_); }
        launch_wb_init(w, o->initial_lambda, s_);
        counts();
        const bool polish = b.mixed && o->fp64_polish;
        const int max_rounds = 2 * std::max(o->max_iterations, 0) + 2;
        for (int round = 0; round < max_rounds; ++round) {
            if (hc[WB_NOT_DONE] == 0) {
                if (!(polish && b.mixed && hc[WB_WANTS_POLISH] > 0)) break;
                // Every window has stopped in FP32: the parked ones continue in FP64.
                b.mixed = 0;
                retry_round_.reset();
                launch_wb_start_polish(w, s_);
            }
            { SFMBA_PHASE(PH_LM); launch_wb_begin_outer(w, o->max_iterations, s_); }
            counts();
            if (hc[WB_NOT_DONE] == 0) continue;
            { SFMBA_PHASE(PH_LM); launch_wb_live(b, w, false, s_); }
            {
                SFMBA_PHASE(PH_LINEARIZE);
                launch_prepare_images(b, s_);
                launch_linearize(b, s_);
            }
            { SFMBA_PHASE(PH_POINT_REDUCE); launch_point_reduce(b, s_); }
            { SFMBA_PHASE(PH_IMAGE_REDUCE); launch_image_blocks_records(b, s_); launch_diag_fold(b, s_); }
            for (int inner = 0; inner < kMaxDampingRetries; ++inner) {
                // One retry round of every window, the same launches each round
                // (the windows taking part are flagged on the device). The Schur
                // reduction's launch shape is tuned at the first round of the
                // process for this block width and size (run eagerly: the round is
                // captured as a graph only from its second use).
                int vs = -1;
                auto round = [&] {
                    { SFMBA_PHASE(PH_LM); launch_wb_begin_retry(w, s_); launch_wb_live(b, w, true, s_); }
                    { SFMBA_PHASE(PH_POINT_INVERSE); launch_wb_point_inverse(b, w, s_); }
                    { SFMBA_PHASE(PH_IMAGE_RHS); launch_image_rhs(b, s_); launch_fold_rhs(b, s_); }
                    {
                        SFMBA_PHASE(PH_SCHUR);
                        if (vs < 0) {
                            vs = o->kernel_variant > 0 ? (o->kernel_variant - 1) % kWbSchurVariants
                                                       : tuned_variant(ctx_.device, b.mixed ? 2 : 3, kWbSchurVariants,
                                                                       b, s_, [&](int v) { launch_wb_schur(b, w, s_, v); });
                        }
                        launch_wb_schur(b, w, s_, vs);
                    }
                    { SFMBA_PHASE(PH_FOLD); launch_wb_fold(b, w, s_); }
                    { SFMBA_PHASE(PH_CHOLESKY); launch_wb_cholesky(b, w, s_); }
                    { SFMBA_PHASE(PH_TRSV); launch_wb_solve(b, w, w.rhs_p, b.work2, s_); }
                    if (b.mixed) {
                        SFMBA_PHASE(PH_REFINE);
                        for (int k = 0; k < o->refinement_steps; ++k) launch_wb_refine(b, w, s_);
                    }
                    { SFMBA_PHASE(PH_TRSV); launch_wb_scatter(b, w, s_); }
                    { SFMBA_PHASE(PH_BACKSUB); launch_backsub_update(b, b.delta, s_); }
                    { SFMBA_PHASE(PH_COST); launch_wb_cost(b, w, true, s_); }
                    { SFMBA_PHASE(PH_LM); launch_wb_accept_commit(b, w, s_); }
                    launch_wb_summary(w, s_);
                    SFMBA_CUDA(cudaMemcpyAsync(hc, w.counts, 4 * sizeof(int), cudaMemcpyDeviceToHost, s_));
                };
                retry_round_.run(s_, !profiler().on, round);
                SFMBA_CUDA(cudaStreamSynchronize(s_));
                if (hc[WB_FACTOR_FAILED] > 0) {
                    // LU fallback for the windows whose Cholesky failed (lib.rs:1084-1092)
                    {
                        SFMBA_PHASE(PH_LU);
                        launch_wb_lu(b, w, hc[WB_FACTOR_FAILED], s_);
                        launch_wb_scatter(b, w, s_);
                    }
                    { SFMBA_PHASE(PH_BACKSUB); launch_backsub_update(b, b.delta, s_); }
                    { SFMBA_PHASE(PH_COST); launch_wb_cost(b, w, true, s_); }
                    { SFMBA_PHASE(PH_LM); launch_wb_accept_commit(b, w, s_); launch_wb_reject_failed(w, s_); }
                    counts();
                }
                if (hc[WB_RETRY_PENDING] == 0) break;
            }
            { SFMBA_PHASE(PH_LM); launch_wb_end_outer(w, o->max_iterations, polish && b.mixed, o->target_cost, s_); }
            counts();
        }
        std::vector<WinState> ws(w.W);
        SFMBA_CUDA(cudaMemcpyAsync(ws.data(), w.ws, sizeof(WinState) * w.W, cudaMemcpyDeviceToHost, s_));
        SFMBA_CUDA(cudaStreamSynchronize(s_));
        return ws;
    }

    // Window results in the callers' buffers (host), points back in each
    // window's own order.
    void copy_out_batched(const Batch &B, sfmba_result *res) {
        const Bufs &b = b_;
        scatter_points(b.points, b.pt_old2new, b.nP, b.points_trial, s_);
        std::vector<double> poses((size_t)b.nI * 7), points((size_t)b.nP * 3), cams((size_t)b.nC * 8);
        if (!poses.empty())
            SFMBA_CUDA(cudaMemcpyAsync(poses.data(), b.poses, sizeof(double) * poses.size(), cudaMemcpyDeviceToHost, s_));
        if (!points.empty())
            SFMBA_CUDA(cudaMemcpyAsync(points.data(), b.points_trial, sizeof(double) * points.size(),
                                       cudaMemcpyDeviceToHost, s_));
        if (!cams.empty())
            SFMBA_CUDA(cudaMemcpyAsync(cams.data(), b.cams, sizeof(double) * cams.size(), cudaMemcpyDeviceToHost, s_));
        SFMBA_CUDA(cudaStreamSynchronize(s_));
        for (int w = 0; w < B.W; ++w) {
            const sfmba_problem &p = B.window(w);
            sfmba_result &r = res[w];
            if (r.poses && p.num_images)
                std::memcpy(r.poses, poses.data() + (size_t)B.img_base[w] * 7, sizeof(double) * 7 * p.num_images);
            if (r.points && p.num_points)
                std::memcpy(r.points, points.data() + (size_t)B.pt_base[w] * 3, sizeof(double) * 3 * p.num_points);
            if (r.camera_params && p.num_cameras)
                std::memcpy(r.camera_params, cams.data() + (size_t)B.cam_base[w] * 8,
                            sizeof(double) * 8 * p.num_cameras);
        }
    }

    void copy_out(sfmba_result *r, bool device) {
        const cudaMemcpyKind k = device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
        if (r->poses && b_.nI)
            SFMBA_CUDA(cudaMemcpyAsync(r->poses, b_.poses, sizeof(double) * 7 * (size_t)b_.nI, k, s_));
        if (r->points && b_.nP) {
            const double *src = b_.points;
            if (b_.pt_old2new) {  // back to the caller's point order
                scatter_points(b_.points, b_.pt_old2new, b_.nP, b_.points_trial, s_);
                src = b_.points_trial;
            }
            SFMBA_CUDA(cudaMemcpyAsync(r->points, src, sizeof(double) * 3 * (size_t)b_.nP, k, s_));
        }
        if (r->camera_params && b_.nC)
            SFMBA_CUDA(cudaMemcpyAsync(r->camera_params, b_.cams, sizeof(double) * 8 * (size_t)b_.nC, k, s_));
        SFMBA_CUDA(cudaStreamSynchronize(s_));
    }

    const Bufs &bufs() const { return b_; }

  private:
    Context &ctx_;
    cudaStream_t s_;
    Bufs b_;
    WinBufs w_;
    Layout lay_;
    Replay pcg_chunk_[2], retry_round_;  // PCG chunk without / with the coarse correction
    bool coarse_valid_ = false;  // the coarse inverse in b_.co.Ainv is usable
    double coarse_lambda_ = 0.0;
    int coarse_outer_ = 0;
    int solver_ = SFMBA_SOLVER_DENSE;
};

int fail(const Error &e) {
    g_last_error = e.what();
    return e.status;
}

template <typename F>
int guarded(F &&f) {
    try {
        g_last_error.clear();
        f();
        return SFMBA_OK;
    } catch (const Error &e) {
        return fail(e);
    } catch (const std::exception &e) {
        g_last_error = e.what();
        return SFMBA_ERR_INTERNAL;
    }
}

int bundle_adjust_impl(const sfmba_problem *p, const sfmba_options *o, sfmba_result *r, bool device,
                       void *stream) {
    return guarded([&] {
        const double t0 = now_s();
        if (!r) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "result is NULL");
        check_options(o);
        check_problem_shape(p);
        if (!device) check_problem_host(p);
        Context &ctx = context();
        cudaStream_t s = (device && stream) ? (cudaStream_t)stream : ctx.stream;
        Solver solver(ctx, s);
        {
            PhaseScope ps(PH_SETUP, s);
            solver.setup(p, o, device, true);
        }
        SolveOutput out = solver.run(o);
        solver.copy_out(r, device);
        profiler().resolve();
        r->initial_cost = out.initial_cost;
        r->final_cost = out.final_cost;
        r->iterations_run = out.iterations;
        r->damping_retries = out.retries;
        r->solver_used = out.solver;
        r->polish_iteration = out.polish_iteration;
        r->linear_iterations = out.linear_iterations;
        r->reduced_dim = out.n;
        r->valid_observations = out.valid_obs;
        r->status = SFMBA_OK;
        r->seconds = now_s() - t0;
    });
}

}  // namespace

// Sets the message sfmba_last_error() returns on this thread.
void record_error(const char *message) { g_last_error = message; }

}  // namespace sfmba

using namespace sfmba;

extern "C" {

void sfmba_default_options(sfmba_options *o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->max_iterations = 50;
    o->initial_lambda = 1e-3;
    o->robust_loss = SFMBA_LOSS_HUBER;
    o->loss_scale_px = 2.0;
    o->precision = SFMBA_PRECISION_FP64;
    o->solver = SFMBA_SOLVER_AUTO;
    o->pcg_max_iterations = 100;
    o->pcg_tolerance = 0.1;
    o->refinement_steps = 1;
    o->target_cost = 0.0;
    o->dense_max_dim = 6000;
    o->fp64_polish = 0;
}

int sfmba_bundle_adjust(const sfmba_problem *p, const sfmba_options *o, sfmba_result *r) {
    int st = bundle_adjust_impl(p, o, r, false, nullptr);
    if (r) r->status = st;
    return st;
}

int sfmba_bundle_adjust_device(const sfmba_problem *p, const sfmba_options *o, sfmba_result *r,
                               void *stream) {
    int st = bundle_adjust_impl(p, o, r, true, stream);
    if (r) r->status = st;
    return st;
}

static int cost_entry(const sfmba_problem *p, const sfmba_options *o, double *out, int mode) {
    return guarded([&] {
        if (!out) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "output is NULL");
        check_problem_shape(p);
        check_problem_host(p);
        sfmba_options opt;
        sfmba_default_options(&opt);
        if (o) opt = *o;
        check_options(&opt);
        Context &ctx = context();
        Solver solver(ctx, ctx.stream);
        solver.setup(p, &opt, false, false);
        const Bufs &b = solver.bufs();
        if (mode == 0) launch_cost(b, false, false, ctx.stream);
        else launch_mean_error(b, ctx.stream);
        solver.read_state();
        const LMState &hs = *ctx.h_state;
        if (mode == 0) *out = hs.cost;
        else *out = hs.trial_valid_obs == 0 ? 0.0 : hs.trial_cost / (double)hs.trial_valid_obs;
    });
}

int sfmba_total_cost(const sfmba_problem *p, const sfmba_options *o, double *out) {
    return cost_entry(p, o, out, 0);
}

int sfmba_mean_reprojection_error(const sfmba_problem *p, double *out) {
    return cost_entry(p, nullptr, out, 1);
}

int sfmba_default_fixed_params_mask(int64_t n, const int32_t *models, uint8_t *out) {
    return guarded([&] {
        if (n < 0 || (n > 0 && (!models || !out))) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "bad arguments");
        for (int64_t c = 0; c < n; ++c) {
            const int m = models[c];
            if (model_dof(m) == 0) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "unknown camera model id");
            std::memset(out + c * 8, 0, 8);
            // intrinsics.rs:33-43: principal point is (1,2) for the f-only models, (2,3) otherwise
            const int a = (m == SFMBA_SIMPLE_PINHOLE || m == SFMBA_SIMPLE_RADIAL || m == SFMBA_RADIAL) ? 1 : 2;
            out[c * 8 + a] = 1;
            out[c * 8 + a + 1] = 1;
        }
    });
}

int sfmba_residuals_jacobians(const sfmba_problem *p, int32_t precision, double *r, double *j_pose,
                              double *j_point, double *j_camera, uint8_t *valid) {
    return guarded([&] {
        check_problem_shape(p);
        check_problem_host(p);
        if (precision != SFMBA_PRECISION_FP64 && precision != SFMBA_PRECISION_MIXED)
            throw Error(SFMBA_ERR_INVALID_ARGUMENT, "unknown precision");
        const long long nO = p->num_observations;
        const int nI = (int)p->num_images, nC = (int)p->num_cameras, nP = (int)p->num_points;
        Context &ctx = context();
        cudaStream_t s = ctx.stream;
        Arena &A = ctx.main;
        JacProbe q{};
        for (int pass = 0; pass < 2; ++pass) {
            if (pass == 0) A.begin_sizing(); else A.commit();
            q.poses = A.take<double>((size_t)nI * 7);
            q.cams = A.take<double>((size_t)nC * 8);
            q.cam_of_img = A.take<int>(nI);
            q.cam_model = A.take<int>(nC);
            q.points = A.take<double>((size_t)nP * 3);
            q.obs_img = A.take<int>(nO);
            q.obs_pt = A.take<int>(nO);
            q.obs_xy = A.take<double>((size_t)nO * 2);
            q.r = A.take<double>((size_t)nO * 2);
            q.jp = A.take<double>((size_t)nO * 12);
            q.jx = A.take<double>((size_t)nO * 6);
            q.jc = A.take<double>((size_t)nO * 16);
            q.valid = A.take<unsigned char>(nO);
        }
        q.nO = nO;
        put(q.poses, p->poses, (size_t)nI * 7, false, s);
        put(q.cams, p->camera_params, (size_t)nC * 8, false, s);
        put(q.cam_of_img, p->camera_of_image, nI, false, s);
        put(q.cam_model, p->camera_model, nC, false, s);
        put(q.points, p->points, (size_t)nP * 3, false, s);
        put(q.obs_img, p->obs_image, nO, false, s);
        put(q.obs_pt, p->obs_point, nO, false, s);
        put(q.obs_xy, p->obs_xy, (size_t)nO * 2, false, s);
        launch_jacobian_probe(q, precision == SFMBA_PRECISION_MIXED, s);
        auto get = [&](void *dst, const void *src, size_t bytes) {
            if (dst && bytes) SFMBA_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s));
        };
        get(r, q.r, sizeof(double) * 2 * nO);
        get(j_pose, q.jp, sizeof(double) * 12 * nO);
        get(j_point, q.jx, sizeof(double) * 6 * nO);
        get(j_camera, q.jc, sizeof(double) * 16 * nO);
        get(valid, q.valid, nO);
        SFMBA_CUDA(cudaStreamSynchronize(s));
    });
}

int sfmba_filter_and_reoptimize(const sfmba_problem *p, const sfmba_options *o, double threshold_px,
                                sfmba_result *r, uint8_t *keep_out) {
    const int st = guarded([&] {
        const double t0 = now_s();
        if (!r) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "result is NULL");
        check_options(o);
        check_problem_shape(p);
        check_problem_host(p);
        if (std::isnan(threshold_px)) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "threshold_px is NaN");
        Context &ctx = context();
        cudaStream_t s = ctx.stream;
        const int nI = (int)p->num_images, nC = (int)p->num_cameras, nP = (int)p->num_points;
        const long long nO = p->num_observations;
        Arena &A = ctx.aux;
        double *poses[2], *cams[2], *points[2];
        int *cam_of_img = nullptr, *cam_model = nullptr;
        uint8_t *fpose = nullptr, *fcam = nullptr, *fcp = nullptr;
        unsigned char *keep = nullptr;
        FilterBufs f;
        const size_t tb = filter_temp_bytes(nO);
        for (int pass = 0; pass < 2; ++pass) {
            if (pass == 0) A.begin_sizing(); else A.commit();
            for (int k = 0; k < 2; ++k) {
                poses[k] = A.take<double>((size_t)nI * 7);
                cams[k] = A.take<double>((size_t)nC * 8);
                points[k] = A.take<double>((size_t)nP * 3);
                f.img[k] = A.take<int>(nO);
                f.pt[k] = A.take<int>(nO);
                f.xy[k] = A.take<double>((size_t)nO * 2);
                f.orig[k] = A.take<int>(nO);
            }
            cam_of_img = A.take<int>(nI);
            cam_model = A.take<int>(nC);
            fpose = p->fixed_poses ? A.take<uint8_t>(nI) : nullptr;
            fcam = p->fixed_cameras ? A.take<uint8_t>(nC) : nullptr;
            fcp = p->fixed_camera_params ? A.take<uint8_t>((size_t)nC * 8) : nullptr;
            keep = A.take<unsigned char>(nO);
            f.flag = A.take<unsigned char>(nO);
            f.sel = A.take<int>(nO);
            f.iota = A.take<int>(nO);
            f.count = A.take<int>(1);
            f.temp = A.take<char>(tb);
        }
        f.temp_bytes = tb;
        f.cam_of_img = cam_of_img;
        f.cam_model = cam_model;
        put(cam_of_img, p->camera_of_image, nI, false, s);
        put(cam_model, p->camera_model, nC, false, s);
        put(poses[0], p->poses, (size_t)nI * 7, false, s);
        put(cams[0], p->camera_params, (size_t)nC * 8, false, s);
        put(points[0], p->points, (size_t)nP * 3, false, s);
        put(f.img[0], p->obs_image, nO, false, s);
        put(f.pt[0], p->obs_point, nO, false, s);
        put(f.xy[0], p->obs_xy, (size_t)nO * 2, false, s);
        if (fpose) put(fpose, p->fixed_poses, nI, false, s);
        if (fcam) put(fcam, p->fixed_cameras, nC, false, s);
        if (fcp) put(fcp, p->fixed_camera_params, (size_t)nC * 8, false, s);
        launch_filter_iota(f.orig[0], nO, s);
        launch_filter_iota(f.iota, nO, s);
        // The adjustments run on these device arrays: input parameters in one
        // set, output in the other; observations in filter set 0.
        sfmba_problem dp{};
        dp.num_images = nI; dp.num_cameras = nC; dp.num_points = nP;
        dp.camera_of_image = cam_of_img; dp.camera_model = cam_model;
        dp.fixed_poses = fpose; dp.fixed_cameras = fcam; dp.fixed_camera_params = fcp;
        sfmba_result dr{};
        int cur = 0;  // parameter set of the next adjustment's input
        long long m = nO;
        auto adjust = [&] {
            dp.poses = poses[cur]; dp.camera_params = cams[cur]; dp.points = points[cur];
            dp.num_observations = m; dp.obs_image = f.img[0]; dp.obs_point = f.pt[0]; dp.obs_xy = f.xy[0];
            dr.poses = poses[cur ^ 1]; dr.camera_params = cams[cur ^ 1]; dr.points = points[cur ^ 1];
            const int s2 = bundle_adjust_impl(&dp, o, &dr, true, s);
            if (s2 != SFMBA_OK) throw Error(s2, g_last_error);
            cur ^= 1;  // the output is the next input
        };
        adjust();
        for (int round = 0; round < 2; ++round) {  // FILTER_ROUNDS (lib.rs:1735)
            launch_filter_select(f, m, poses[cur], cams[cur], points[cur], threshold_px, s);
            int kept = 0;
            SFMBA_CUDA(cudaMemcpyAsync(&kept, f.count, sizeof(int), cudaMemcpyDeviceToHost, s));
            SFMBA_CUDA(cudaStreamSynchronize(s));
            if (kept == m || kept < 12) break;  // MIN_OBSERVATIONS (lib.rs:1736)
            std::swap(f.img[0], f.img[1]);
            std::swap(f.pt[0], f.pt[1]);
            std::swap(f.xy[0], f.xy[1]);
            std::swap(f.orig[0], f.orig[1]);
            m = kept;
            adjust();
        }
        if (r->poses && nI)
            SFMBA_CUDA(cudaMemcpyAsync(r->poses, poses[cur], sizeof(double) * 7 * nI, cudaMemcpyDeviceToHost, s));
        if (r->points && nP)
            SFMBA_CUDA(cudaMemcpyAsync(r->points, points[cur], sizeof(double) * 3 * nP, cudaMemcpyDeviceToHost, s));
        if (r->camera_params && nC)
            SFMBA_CUDA(cudaMemcpyAsync(r->camera_params, cams[cur], sizeof(double) * 8 * nC, cudaMemcpyDeviceToHost,
                                       s));
        if (keep_out && nO) {
            launch_filter_keep(f.orig[0], m, keep, nO, s);
            SFMBA_CUDA(cudaMemcpyAsync(keep_out, keep, (size_t)nO, cudaMemcpyDeviceToHost, s));
        }
        SFMBA_CUDA(cudaStreamSynchronize(s));
        r->initial_cost = dr.initial_cost;
        r->final_cost = dr.final_cost;
        r->iterations_run = dr.iterations_run;
        r->damping_retries = dr.damping_retries;
        r->solver_used = dr.solver_used;
        r->polish_iteration = dr.polish_iteration;
        r->linear_iterations = dr.linear_iterations;
        r->reduced_dim = dr.reduced_dim;
        r->valid_observations = dr.valid_observations;
        r->seconds = now_s() - t0;
    });
    if (r) r->status = st;
    return st;
}

namespace {

// CameraModel::opencv_distortion (crates/sfm-core/src/camera.rs:192-200):
// the distortion coefficients of `params` in OpenCV order, zero where the
// model has none.
void opencv_distortion(int model, const double *c, double out[6]) {
    for (int k = 0; k < 6; ++k) out[k] = 0.0;
    switch (model) {
    case SFMBA_SIMPLE_RADIAL: out[0] = c[3]; break;
    case SFMBA_RADIAL: out[0] = c[3]; out[1] = c[4]; break;
    case SFMBA_OPENCV: out[0] = c[4]; out[1] = c[5]; out[2] = c[6]; out[3] = c[7]; break;
    case SFMBA_OPENCV_FISHEYE: out[0] = c[4]; out[1] = c[5]; out[4] = c[6]; out[5] = c[7]; break;
    default: break;
    }
}

// One candidate of the global adjustment, in host buffers.
struct Candidate {
    std::vector<double> poses, points, cams;
    std::vector<uint8_t> keep;
    sfmba_result r{};
    double mean_error = std::numeric_limits<double>::quiet_NaN();
};

}  // namespace

int sfmba_adjust_global(const sfmba_problem *p, const sfmba_options *o, int32_t mode, double threshold_px,
                        sfmba_result *r, uint8_t *keep_out, int32_t *chose_free_out, double *mean_errors_out) {
    const int st = guarded([&] {
        const double t0 = now_s();
        if (!r) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "result is NULL");
        if (mode != SFMBA_INTRINSICS_FIXED && mode != SFMBA_INTRINSICS_FREE && mode != SFMBA_INTRINSICS_FREE_GUARDED)
            throw Error(SFMBA_ERR_INVALID_ARGUMENT, "unknown intrinsics mode");
        check_options(o);
        check_problem_shape(p);
        check_problem_host(p);
        const int nI = (int)p->num_images, nC = (int)p->num_cameras, nP = (int)p->num_points;
        const long long nO = p->num_observations;
        // Images per camera (lib.rs:1639-1642) and the cameras left free when
        // intrinsics are free: seen by >= 5 images and not fixed by the user
        // (:1601-1611, :1648-1657).
        std::vector<int> per_cam(nC, 0);
        for (int i = 0; i < nI; ++i) per_cam[p->camera_of_image[i]] += 1;
        constexpr int kMinImagesPerCamera = 5;
        std::vector<uint8_t> all_fixed(nC, 1), free_fixed(nC, 0);
        bool any_eligible = false;
        for (int c = 0; c < nC; ++c) {
            const bool user = p->fixed_cameras && p->fixed_cameras[c];
            free_fixed[c] = (per_cam[c] < kMinImagesPerCamera || user) ? 1 : 0;
            any_eligible = any_eligible || per_cam[c] >= kMinImagesPerCamera;
        }
        // run_ba (:1585-1593): the filtered adjustment in the guarded mode,
        // the plain one otherwise.
        auto run = [&](const std::vector<uint8_t> &fixed_cams, Candidate &out) {
            sfmba_problem q = *p;
            q.fixed_cameras = fixed_cams.data();
            out.poses.assign((size_t)nI * 7, 0.0);
            out.points.assign((size_t)nP * 3, 0.0);
            out.cams.assign((size_t)nC * 8, 0.0);
            out.keep.assign((size_t)nO, 1);
            out.r = sfmba_result{};
            out.r.poses = out.poses.data();
            out.r.points = out.points.data();
            out.r.camera_params = out.cams.data();
            const int s2 = mode == SFMBA_INTRINSICS_FREE_GUARDED
                               ? sfmba_filter_and_reoptimize(&q, o, threshold_px, &out.r, out.keep.data())
                               : sfmba_bundle_adjust(&q, o, &out.r);
            if (s2 != SFMBA_OK) throw Error(s2, g_last_error);
        };
        // eval_error (:1567-1578): plain mean reprojection error of the
        // output over all the problem's observations.
        auto eval_error = [&](Candidate &c) {
            sfmba_problem q = *p;
            q.poses = c.poses.data();
            q.points = c.points.data();
            q.camera_params = c.cams.data();
            q.fixed_poses = nullptr;
            q.fixed_cameras = nullptr;
            q.fixed_camera_params = nullptr;
            const int s2 = sfmba_mean_reprojection_error(&q, &c.mean_error);
            if (s2 != SFMBA_OK) throw Error(s2, g_last_error);
        };
        Candidate fixed, free;
        Candidate *chosen = nullptr;
        if (mode == SFMBA_INTRINSICS_FREE) {  // :1598-1621, no comparison
            run(free_fixed, free);
            chosen = &free;
        } else {
            run(all_fixed, fixed);
            chosen = &fixed;
            if (mode == SFMBA_INTRINSICS_FREE_GUARDED && any_eligible) {
                run(free_fixed, free);
                bool plausible = true;  // :1672-1677
                for (int c = 0; c < nC; ++c) {
                    double d[6];
                    opencv_distortion(p->camera_model[c], free.cams.data() + 8 * (size_t)c, d);
                    for (int k = 0; k < 6; ++k) plausible = plausible && std::fabs(d[k]) < 0.5;
                }
                eval_error(fixed);
                eval_error(free);
                if (plausible && free.mean_error < fixed.mean_error) chosen = &free;  // :1691-1695
            }
        }
        if (r->poses) std::memcpy(r->poses, chosen->poses.data(), sizeof(double) * 7 * (size_t)nI);
        if (r->points) std::memcpy(r->points, chosen->points.data(), sizeof(double) * 3 * (size_t)nP);
        if (r->camera_params) std::memcpy(r->camera_params, chosen->cams.data(), sizeof(double) * 8 * (size_t)nC);
        if (keep_out && nO) std::memcpy(keep_out, chosen->keep.data(), (size_t)nO);
        if (chose_free_out) *chose_free_out = chosen == &free ? 1 : 0;
        if (mean_errors_out) {
            mean_errors_out[0] = fixed.mean_error;
            mean_errors_out[1] = free.mean_error;
        }
        double *pp = r->poses, *pt = r->points, *pc = r->camera_params;
        *r = chosen->r;
        r->poses = pp; r->points = pt; r->camera_params = pc;
        r->seconds = now_s() - t0;
    });
    if (r) r->status = st;
    return st;
}

namespace {

// Offsets of a batch of correspondence sets: 0 first, non-decreasing.
long long check_offsets(int32_t num, const int64_t *offsets) {
    if (num < 0) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "negative batch size");
    if (num > 0 && !offsets) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "offsets is NULL");
    if (num == 0) return 0;
    if (offsets[0] != 0) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "offsets[0] must be 0");
    for (int32_t k = 0; k < num; ++k)
        if (offsets[k + 1] < offsets[k]) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "offsets decrease");
    return offsets[num];
}

}  // namespace

int sfmba_refine_pose_gauss_newton_batched(int32_t num, const int64_t *offsets, const double *points3d,
                                           const double *points2d_norm, int32_t iterations, double *poses) {
    return guarded([&] {
        const long long N = check_offsets(num, offsets);
        if (iterations < 0) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "negative iteration count");
        if (num > 0 && !poses) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "poses is NULL");
        if (N > 0 && (!points3d || !points2d_norm)) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "points are NULL");
        if (num == 0) return;
        Context &ctx = context();
        cudaStream_t s = ctx.stream;
        Arena &A = ctx.aux;
        long long *off = nullptr;
        double *X = nullptr, *uv = nullptr, *P = nullptr;
        for (int pass = 0; pass < 2; ++pass) {
            if (pass == 0) A.begin_sizing(); else A.commit();
            off = A.take<long long>((size_t)num + 1);
            X = A.take<double>((size_t)N * 3 + 1);
            uv = A.take<double>((size_t)N * 2 + 1);
            P = A.take<double>((size_t)num * 7);
        }
        put(off, reinterpret_cast<const long long *>(offsets), (size_t)num + 1, false, s);
        if (N) {
            put(X, points3d, (size_t)N * 3, false, s);
            put(uv, points2d_norm, (size_t)N * 2, false, s);
        }
        put(P, poses, (size_t)num * 7, false, s);
        launch_refine_pose_gn(off, X, uv, num, iterations, P, s);
        SFMBA_CUDA(cudaMemcpyAsync(poses, P, sizeof(double) * 7 * (size_t)num, cudaMemcpyDeviceToHost, s));
        SFMBA_CUDA(cudaStreamSynchronize(s));
    });
}

int sfmba_pnp_ransac_batched(int32_t num, const int64_t *offsets, const double *points3d,
                             const double *points2d_norm, double threshold, int32_t max_iterations,
                             double *poses_out, uint8_t *inliers_out, int32_t *found_out, int64_t *iterations_out) {
    return guarded([&] {
        const long long N = check_offsets(num, offsets);
        if (max_iterations < 0) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "negative max_iterations");
        if (std::isnan(threshold)) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "threshold is NaN");
        if (num > 0 && (!poses_out || !found_out)) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "outputs are NULL");
        if (N > 0 && (!points3d || !points2d_norm)) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "points are NULL");
        if (num == 0) return;
        if ((long long)num * 32 > (1LL << 31) - 1) throw Error(SFMBA_ERR_UNSUPPORTED, "too many images");
        Context &ctx = context();
        cudaStream_t s = ctx.stream;
        Arena &A = ctx.aux;
        PnpBufs q;
        q.P = num;
        q.max_it = max_iterations;
        // Hypotheses per image per round: at most kMaxRound; the first round
        // takes 64 (the pipeline's usual inlier ratios end the loop within
        // ~60 iterations), later rounds what the longest remaining loop needs.
        constexpr int kMaxRound = 128;
        const int b_cap = (int)std::max<long long>(1, std::min<long long>(kMaxRound, max_iterations));
        q.B = b_cap;
        q.thr = threshold;
        long long *off = nullptr, *iters = nullptr;
        double *X = nullptr, *uv = nullptr;
        unsigned long long *raw = nullptr;
        for (int pass = 0; pass < 2; ++pass) {
            if (pass == 0) A.begin_sizing(); else A.commit();
            off = A.take<long long>((size_t)num + 1);
            X = A.take<double>((size_t)N * 3 + 1);
            uv = A.take<double>((size_t)N * 2 + 1);
            raw = A.take<unsigned long long>((size_t)6 * max_iterations + 1);
            q.state = A.take<char>(pnp_state_bytes() * (size_t)num);
            q.models = A.take<double>((size_t)num * q.B * 8);
            q.valid = A.take<unsigned char>((size_t)num * q.B);
            q.counts = A.take<long long>((size_t)num * q.B);
            q.active = A.take<int>(2);
            q.dlt_scratch = A.take<double>((size_t)N * 24 + 1);
            q.slot_scratch = A.take<long long>((size_t)N + 1);
            q.mask = A.take<unsigned char>((size_t)N + 1);
            q.mask_trial = A.take<unsigned char>((size_t)N + 1);
            q.poses = A.take<double>((size_t)num * 7);
            q.found = A.take<int>(num);
            iters = A.take<long long>(num);
        }
        q.off = off;
        q.X = X;
        q.uv = uv;
        q.raw = raw;
        // ransac.rs:43-60: xorshift64 seeded 0xFACADE | 1, six values per iteration.
        std::vector<unsigned long long> stream((size_t)6 * max_iterations);
        unsigned long long x = 0xFACADEull | 1ull;
        for (auto &v : stream) {
            x ^= x << 13;
            x ^= x >> 7;
            x ^= x << 17;
            v = x;
        }
        put(off, reinterpret_cast<const long long *>(offsets), (size_t)num + 1, false, s);
        if (N) {
            put(X, points3d, (size_t)N * 3, false, s);
            put(uv, points2d_norm, (size_t)N * 2, false, s);
        }
        if (!stream.empty()) put_vec(raw, stream, s);
        launch_pnp_init(q, s);
        int round = std::min(b_cap, 64);
        for (long long base = 0; base < max_iterations;) {
            q.B = round;
            launch_pnp_round(q, base, s);
            base += round;
            int act[2] = {0, 0};
            SFMBA_CUDA(cudaMemcpyAsync(act, q.active, sizeof(act), cudaMemcpyDeviceToHost, s));
            SFMBA_CUDA(cudaStreamSynchronize(s));
            if (act[0] == 0) break;
            round = std::min(b_cap, std::max(8, (act[1] + 7) / 8 * 8));
        }
        launch_pnp_finish(q, s);
        launch_pnp_iterations(q, iters, s);
        std::vector<int> found(num);
        SFMBA_CUDA(cudaMemcpyAsync(poses_out, q.poses, sizeof(double) * 7 * (size_t)num, cudaMemcpyDeviceToHost, s));
        SFMBA_CUDA(cudaMemcpyAsync(found.data(), q.found, sizeof(int) * (size_t)num, cudaMemcpyDeviceToHost, s));
        if (inliers_out && N)
            SFMBA_CUDA(cudaMemcpyAsync(inliers_out, q.mask, (size_t)N, cudaMemcpyDeviceToHost, s));
        if (iterations_out)
            SFMBA_CUDA(cudaMemcpyAsync(iterations_out, iters, sizeof(long long) * (size_t)num,
                                       cudaMemcpyDeviceToHost, s));
        SFMBA_CUDA(cudaStreamSynchronize(s));
        for (int32_t k = 0; k < num; ++k) found_out[k] = found[k];
    });
}

int sfmba_colmap_model_stats(const char *dir, int64_t *counts, double *mean_error) {
    return guarded([&] {
        if (!dir) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "dir is NULL");
        const ColmapModel m = colmap_read(dir);
        if (counts) {
            long long track = 0, kp = 0;
            for (const auto &kv : m.points) track += (long long)kv.second.track.size();
            for (const auto &kv : m.images) kp += (long long)kv.second.keypoints.size();
            counts[0] = (int64_t)m.cameras.size();
            counts[1] = (int64_t)m.images.size();
            counts[2] = (int64_t)m.points.size();
            counts[3] = track;
            counts[4] = kp;
        }
        if (mean_error) *mean_error = m.mean_reprojection_error();
    });
}

int sfmba_colmap_rewrite(const char *dir_in, const char *dir_out) {
    return guarded([&] {
        if (!dir_in || !dir_out) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "dir is NULL");
        colmap_write(colmap_read(dir_in), dir_out);
    });
}

int sfmba_colmap_refine(const char *dir_in, const char *dir_out, const sfmba_options *o, int32_t refine_intrinsics,
                        sfmba_refine_report *rep) {
    return guarded([&] {
        const double t0 = now_s();
        if (!dir_in || !dir_out) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "dir is NULL");
        sfmba_options opt;
        if (o) {
            opt = *o;
        } else {  // cmd_refine's BaParams (main.rs:1049-1057): Huber, 200 iterations
            sfmba_default_options(&opt);
            opt.robust_loss = SFMBA_LOSS_HUBER;
            opt.max_iterations = 200;
        }
        check_options(&opt);
        ColmapModel m = colmap_read(dir_in);
        if (m.images.size() < 2)
            throw Error(SFMBA_ERR_INVALID_ARGUMENT, "need at least 2 registered images in " + std::string(dir_in));
        if (m.points.empty()) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "no 3D points in " + std::string(dir_in));
        // Compact indices as cmd_refine (main.rs:969-1035): images in id
        // order, one camera block per physical camera in first-use order,
        // points in id order; observations are the track elements whose
        // image and keypoint exist, point by point (the reference walks a
        // hash map here, an order without meaning for the result).
        std::vector<uint32_t> image_ids;
        std::map<uint32_t, int> image_pos;
        for (const auto &kv : m.images) {
            image_pos[kv.first] = (int)image_ids.size();
            image_ids.push_back(kv.first);
        }
        std::vector<uint32_t> camera_id_list;
        std::map<uint32_t, int> camera_index_of;
        std::vector<int32_t> cam_of_img, cam_model;
        std::vector<double> cam_params, poses;
        for (uint32_t id : image_ids) {
            const ColmapImage &im = m.images.at(id);
            auto it = camera_index_of.find(im.camera_id);
            if (it == camera_index_of.end()) {
                auto c = m.cameras.find(im.camera_id);
                if (c == m.cameras.end())
                    throw Error(SFMBA_ERR_INVALID_ARGUMENT, "image " + std::to_string(id) + " uses unknown camera " +
                                                                std::to_string(im.camera_id));
                it = camera_index_of.emplace(im.camera_id, (int)camera_id_list.size()).first;
                camera_id_list.push_back(im.camera_id);
                cam_model.push_back(c->second.model);
                for (double v : c->second.params) cam_params.push_back(v);
            }
            cam_of_img.push_back(it->second);
            for (double v : im.q) poses.push_back(v);
            for (double v : im.t) poses.push_back(v);
        }
        std::vector<uint64_t> point_ids;
        std::vector<double> points;
        std::vector<int32_t> ob_img, ob_pt;
        std::vector<double> ob_xy;
        std::vector<long long> pt_obs{0};
        for (const auto &kv : m.points) {
            const int cp = (int)point_ids.size();
            point_ids.push_back(kv.first);
            for (double v : kv.second.xyz) points.push_back(v);
            for (const auto &te : kv.second.track) {
                auto ip = image_pos.find(te.first);
                if (ip == image_pos.end()) continue;
                const ColmapImage &im = m.images.at(te.first);
                if (te.second >= im.keypoints.size()) continue;
                ob_img.push_back(ip->second);
                ob_pt.push_back(cp);
                ob_xy.push_back((double)im.keypoints[te.second].first);
                ob_xy.push_back((double)im.keypoints[te.second].second);
            }
            pt_obs.push_back((long long)ob_img.size());
        }
        if (ob_img.empty())
            throw Error(SFMBA_ERR_INVALID_ARGUMENT,
                        "no observations linking tracked points to registered images; nothing to refine");
        const int nI = (int)image_ids.size(), nC = (int)camera_id_list.size(), nP = (int)point_ids.size();
        const long long nO = (long long)ob_img.size();
        // Image 0 anchored; cameras fixed, or free with the principal point
        // masked (main.rs:1037-1047).
        std::vector<uint8_t> fixed_poses(nI, 0), fixed_cams(nC, refine_intrinsics ? 0 : 1), fcp((size_t)nC * 8, 0);
        fixed_poses[0] = 1;
        if (refine_intrinsics) {
            const int st = sfmba_default_fixed_params_mask(nC, cam_model.data(), fcp.data());
            if (st != SFMBA_OK) throw Error(st, g_last_error);
        }
        sfmba_problem q{};
        q.num_images = nI; q.num_cameras = nC; q.num_points = nP; q.num_observations = nO;
        q.camera_of_image = cam_of_img.data(); q.camera_model = cam_model.data(); q.camera_params = cam_params.data();
        q.poses = poses.data(); q.points = points.data();
        q.obs_image = ob_img.data(); q.obs_point = ob_pt.data(); q.obs_xy = ob_xy.data();
        q.fixed_poses = fixed_poses.data(); q.fixed_cameras = fixed_cams.data();
        q.fixed_camera_params = refine_intrinsics ? fcp.data() : nullptr;
        const double before = m.mean_reprojection_error();
        std::vector<double> out_poses((size_t)nI * 7), out_points((size_t)nP * 3), out_cams((size_t)nC * 8);
        sfmba_result r{};
        r.poses = out_poses.data(); r.points = out_points.data(); r.camera_params = out_cams.data();
        const int st = sfmba_bundle_adjust(&q, &opt, &r);
        if (st != SFMBA_OK) throw Error(st, g_last_error);
        // Write back (main.rs:1062-1074).
        for (int k = 0; k < nI; ++k) {
            ColmapImage &im = m.images.at(image_ids[k]);
            for (int j = 0; j < 4; ++j) im.q[j] = out_poses[(size_t)k * 7 + j];
            for (int j = 0; j < 3; ++j) im.t[j] = out_poses[(size_t)k * 7 + 4 + j];
        }
        for (int k = 0; k < nP; ++k)
            for (int j = 0; j < 3; ++j) m.points.at(point_ids[k]).xyz[j] = out_points[(size_t)k * 3 + j];
        if (refine_intrinsics)
            for (int c = 0; c < nC; ++c)
                for (int j = 0; j < 8; ++j) m.cameras.at(camera_id_list[c]).params[j] = out_cams[(size_t)c * 8 + j];
        // Each point's error against the refined model, on the device
        // (main.rs:1076-1098): the mean over its observations in front of
        // the camera; a point with none keeps its error.
        {
            Context &ctx = context();
            cudaStream_t s = ctx.stream;
            Arena &A = ctx.aux;
            double *d_poses = nullptr, *d_cams = nullptr, *d_points = nullptr, *d_xy = nullptr, *d_err = nullptr;
            int *d_coi = nullptr, *d_model = nullptr, *d_img = nullptr, *d_n = nullptr;
            long long *d_pt_obs = nullptr;
            for (int pass = 0; pass < 2; ++pass) {
                if (pass == 0) A.begin_sizing(); else A.commit();
                d_poses = A.take<double>((size_t)nI * 7);
                d_cams = A.take<double>((size_t)nC * 8);
                d_points = A.take<double>((size_t)nP * 3);
                d_xy = A.take<double>((size_t)nO * 2);
                d_err = A.take<double>(nP);
                d_coi = A.take<int>(nI);
                d_model = A.take<int>(nC);
                d_img = A.take<int>(nO);
                d_n = A.take<int>(nP);
                d_pt_obs = A.take<long long>((size_t)nP + 1);
            }
            const std::vector<double> &cams_now = refine_intrinsics ? out_cams : cam_params;
            put(d_poses, out_poses.data(), out_poses.size(), false, s);
            put(d_cams, cams_now.data(), cams_now.size(), false, s);
            put(d_points, out_points.data(), out_points.size(), false, s);
            put(d_xy, ob_xy.data(), ob_xy.size(), false, s);
            put_vec(d_coi, cam_of_img, s);
            put_vec(d_model, cam_model, s);
            put_vec(d_img, ob_img, s);
            put_vec(d_pt_obs, pt_obs, s);
            launch_point_errors(d_poses, d_cams, d_points, d_coi, d_model, d_img, d_xy, d_pt_obs, nP, d_err, d_n, s);
            std::vector<double> err(nP);
            std::vector<int> cnt(nP);
            SFMBA_CUDA(cudaMemcpyAsync(err.data(), d_err, sizeof(double) * nP, cudaMemcpyDeviceToHost, s));
            SFMBA_CUDA(cudaMemcpyAsync(cnt.data(), d_n, sizeof(int) * nP, cudaMemcpyDeviceToHost, s));
            SFMBA_CUDA(cudaStreamSynchronize(s));
            for (int k = 0; k < nP; ++k)
                if (cnt[k] > 0) m.points.at(point_ids[k]).error = err[k];
        }
        const double after = m.mean_reprojection_error();
        colmap_write(m, dir_out);
        if (rep) {
            *rep = sfmba_refine_report{};
            rep->num_images = nI;
            rep->num_cameras = nC;
            rep->num_points3d = nP;
            rep->num_observations = nO;
            rep->initial_cost = r.initial_cost;
            rep->final_cost = r.final_cost;
            rep->iterations_run = r.iterations_run;
            rep->mean_error_before_px = before;
            rep->mean_error_after_px = after;
            rep->seconds = now_s() - t0;
        }
    });
}

int sfmba_refine_intrinsics(const sfmba_problem *p, const sfmba_options *o, double *cams) {
    return guarded([&] {
        if (!cams) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "camera_params_inout is NULL");
        check_options(o);
        check_problem_shape(p);
        check_problem_host(p);
        Context &ctx = context();
        cudaStream_t s = ctx.stream;
        const int nI = (int)p->num_images, nC = (int)p->num_cameras, nP = (int)p->num_points;
        const long long nO = p->num_observations;
        // Observations grouped by camera (intrinsics.rs:125-128), in input order.
        std::vector<int> start(nC + 1, 0), list((size_t)nO);
        for (long long k = 0; k < nO; ++k) start[p->camera_of_image[p->obs_image[k]] + 1] += 1;
        for (int c = 0; c < nC; ++c) start[c + 1] += start[c];
        {
            std::vector<int> fill(start.begin(), start.end() - 1);
            for (long long k = 0; k < nO; ++k) list[fill[p->camera_of_image[p->obs_image[k]]]++] = (int)k;
        }
        Arena &A = ctx.aux;
        IntrinsicsBufs q;
        double *poses = nullptr, *points = nullptr, *xy = nullptr, *cam = nullptr;
        int *img = nullptr, *pt = nullptr, *model = nullptr, *cs = nullptr, *cl = nullptr;
        for (int pass = 0; pass < 2; ++pass) {
            if (pass == 0) A.begin_sizing(); else A.commit();
            poses = A.take<double>((size_t)nI * 7);
            points = A.take<double>((size_t)nP * 3);
            xy = A.take<double>((size_t)nO * 2);
            cam = A.take<double>((size_t)nC * 8);
            img = A.take<int>(nO);
            pt = A.take<int>(nO);
            model = A.take<int>(nC);
            cs = A.take<int>((size_t)nC + 1);
            cl = A.take<int>(nO);
        }
        put(poses, p->poses, (size_t)nI * 7, false, s);
        put(points, p->points, (size_t)nP * 3, false, s);
        put(xy, p->obs_xy, (size_t)nO * 2, false, s);
        put(cam, p->camera_params, (size_t)nC * 8, false, s);
        put(img, p->obs_image, nO, false, s);
        put(pt, p->obs_point, nO, false, s);
        put(model, p->camera_model, nC, false, s);
        put_vec(cs, start, s);
        put_vec(cl, list, s);
        q.nC = nC; q.poses = poses; q.points = points; q.ob_xy = xy; q.ob_img = img; q.ob_pt = pt;
        q.cam_model = model; q.cobs_start = cs; q.cobs = cl; q.cams = cam;
        launch_refine_intrinsics(q, o->max_iterations, o->initial_lambda, o->robust_loss, o->loss_scale_px, s);
        if (nC) SFMBA_CUDA(cudaMemcpyAsync(cams, cam, sizeof(double) * 8 * (size_t)nC, cudaMemcpyDeviceToHost, s));
        SFMBA_CUDA(cudaStreamSynchronize(s));
    });
}

int sfmba_bundle_adjust_batched(int32_t num_windows, const sfmba_problem *windows,
                                const sfmba_options *o, sfmba_result *results) {
    const int st = guarded([&] {
        const double t0 = now_s();
        if (num_windows < 0) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "num_windows < 0");
        if (num_windows > 0 && (!windows || !results))
            throw Error(SFMBA_ERR_INVALID_ARGUMENT, "windows or results is NULL");
        check_options(o);
        if (num_windows == 0) return;
        Profiler &prof = profiler();
        double t = now_s();
        for (int w = 0; w < num_windows; ++w) check_problem_shape(&windows[w]);
        parallel_for(num_windows, [&](int w) { check_problem_host(&windows[w]); });
        prof.host("batch_validate", now_s() - t);
        t = now_s();
        Batch B;
        build_batch(num_windows, windows, B);
        prof.host("batch_build", now_s() - t);
        t = now_s();
        Context &ctx = context();
        cudaStream_t s = ctx.stream;
        Solver solver(ctx, s);
        {
            PhaseScope ps(PH_SETUP, s);
            solver.setup(&B.problem, o, false, true, &B);
        }
        SFMBA_CUDA(cudaStreamSynchronize(s));
        prof.host("batch_setup", now_s() - t);
        t = now_s();
        std::vector<WinState> ws = solver.run_batched(o);
        SFMBA_CUDA(cudaStreamSynchronize(s));
        prof.host("batch_solve", now_s() - t);
        t = now_s();
        solver.copy_out_batched(B, results);
        prof.host("batch_copy_out", now_s() - t);
        profiler().resolve();
        const double secs = now_s() - t0;
        for (int w = 0; w < num_windows; ++w) {
            sfmba_result &r = results[w];
            const WinState &x = ws[w];
            r.initial_cost = x.initial_cost;
            r.final_cost = x.cost;
            r.iterations_run = x.iterations;
            r.damping_retries = x.retries;
            r.solver_used = SFMBA_SOLVER_DENSE;
            r.polish_iteration = x.polished && x.polish_iteration >= 0 ? x.polish_iteration : -1;
            r.linear_iterations = 0;
            r.reduced_dim = B.n_w[w];
            r.valid_observations = x.valid_obs;
            r.seconds = secs;
            r.status = SFMBA_OK;
        }
    });
    if (st != SFMBA_OK && results && num_windows > 0)
        for (int w = 0; w < num_windows; ++w) results[w].status = st;
    return st;
}

int sfmba_profile_enable(int32_t on) {
    return guarded([&] {
        Profiler &p = profiler();
        p.reset();
        p.on = on != 0;
        g_kernel_launches = 0;
    });
}

int sfmba_profile_report(char *buf, int64_t len) {
    return guarded([&] {
        Profiler &p = profiler();
        p.resolve();
        std::string js = "{";
        for (int k = 0; k < PH_COUNT; ++k) {
            if (k) js += ",";
            char tmp[160];
            std::snprintf(tmp, sizeof(tmp), "\"%s\":{\"ms\":%.6f,\"launches\":%lld}", kPhaseNames[k], p.ms[k],
                          p.launches[k]);
            js += tmp;
        }
        js += ",\"kernel_launches\":" + std::to_string(g_kernel_launches);
        js += ",\"host_ms\":{";
        bool first = true;
        for (const auto &kv : p.host_ms) {
            char tmp[160];
            std::snprintf(tmp, sizeof(tmp), "%s\"%s\":%.3f", first ? "" : ",", kv.first.c_str(), kv.second);
            js += tmp;
            first = false;
        }
        js += "},\"counts\":{";
        first = true;
        for (const auto &kv : p.counts) {
            js += (first ? "\"" : ",\"") + kv.first + "\":" + std::to_string(kv.second);
            first = false;
        }
        js += "},\"lm_trace\":[";
        for (size_t k = 0; k < p.trace.size(); ++k) js += (k ? "," : "") + p.trace[k];
        js += "]";
        js += ",\"autotune\":" + tune_report() + "}";
        if (!buf || len <= (int64_t)js.size())
            throw Error(SFMBA_ERR_INVALID_ARGUMENT, "profile buffer too small (need " + std::to_string(js.size() + 1) + ")");
        std::memcpy(buf, js.c_str(), js.size() + 1);
    });
}

int sfmba_measure_peaks(double *out) {
    return guarded([&] {
        if (!out) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "out is NULL");
        Context &ctx = context();
        double *sink = nullptr;
        SFMBA_CUDA(cudaMalloc(&sink, sizeof(double)));
        PeakRates r{};
        try {
            r = measure_peaks(ctx.stream, sink);
        } catch (...) {
            cudaFree(sink);
            throw;
        }
        SFMBA_CUDA(cudaFree(sink));
        out[0] = r.dfma_tflops;
        out[1] = r.dmma_tflops;
        out[2] = r.bf16_mma_tflops;
    });
}

int sfmba_dense_cholesky(int64_t n, const double *A, double *L, int32_t tensor_update, double *seconds) {
    return guarded([&] {
        if (n <= 0 || n > 32768) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "n must be in [1, 32768]");
        if (!A || !L) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "A or L is NULL");
        Context &ctx = context();
        cudaStream_t s = ctx.stream;
        Bufs b;
        b.n = (int)n;
        std::vector<void *> owned;
        auto dev_alloc = [&](size_t bytes) {
            void *p = nullptr;
            if (cudaMalloc(&p, bytes) != cudaSuccess) {
                (void)cudaGetLastError();
                for (void *q : owned) cudaFree(q);
                throw Error(SFMBA_ERR_OUT_OF_MEMORY, "device allocation failed");
            }
            owned.push_back(p);
            return p;
        };
        const size_t nn = (size_t)n * n;
        b.L = (double *)dev_alloc(nn * sizeof(double));
        b.Linv = (double *)dev_alloc((size_t)div_up((int)n, kCholNB) * kCholNB * kCholNB * sizeof(double));
        b.state = (LMState *)dev_alloc(sizeof(LMState));
        if (tensor_update) {
            b.oz_slices = (uint16_t *)dev_alloc((size_t)2 * kOzSlices * n * kOzK * sizeof(uint16_t));
            b.oz_exp = (int *)dev_alloc((size_t)2 * n * sizeof(int));
        }
        int failed = 0;
        float ms = 0.0f;
        try {
            SFMBA_CUDA(cudaMemcpyAsync(b.L, A, nn * sizeof(double), cudaMemcpyHostToDevice, s));
            SFMBA_CUDA(cudaMemsetAsync(b.state, 0, sizeof(LMState), s));
            cudaEvent_t e0, e1;
            SFMBA_CUDA(cudaEventCreate(&e0));
            SFMBA_CUDA(cudaEventCreate(&e1));
            SFMBA_CUDA(cudaEventRecord(e0, s));
            launch_cholesky(b, s);
            SFMBA_CUDA(cudaEventRecord(e1, s));
            SFMBA_CUDA(cudaMemcpyAsync(&failed, &b.state->factor_failed, sizeof(int), cudaMemcpyDeviceToHost, s));
            SFMBA_CUDA(cudaMemcpyAsync(L, b.L, nn * sizeof(double), cudaMemcpyDeviceToHost, s));
            SFMBA_CUDA(cudaStreamSynchronize(s));
            SFMBA_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
        } catch (...) {
            for (void *q : owned) cudaFree(q);
            throw;
        }
        for (void *q : owned) cudaFree(q);
        if (failed) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "the matrix is not positive definite");
        for (int64_t r = 0; r < n; ++r)
            for (int64_t c = r + 1; c < n; ++c) L[r * n + c] = 0.0;
        if (seconds) *seconds = ms * 1e-3;
    });
}

const char *sfmba_last_error(void) { return g_last_error.c_str(); }

const char *sfmba_version(void) { return "sfmba-gb300 0.1 (sm_103a)"; }

}  // extern "C"
