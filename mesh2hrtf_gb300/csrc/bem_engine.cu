// bem_engine.cu - host side of the batched Krylov engine: launch table,
// work-item lists, graph capture and replay.
#include <cuda_runtime.h>

#include <cstdlib>
#include <cstring>

#include <cudaTypedefs.h>

#include "bem_engine.h"

namespace bem {

namespace {
// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library)
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        else
            cudaGetLastError();
    }
    return fn;
}

// TMA map of a complex64 matrix viewed as n rows of 2 n floats (row pitch
// 2 lda floats): boxes of 32 floats x kUmRows rows with the 128-byte swizzle,
// zeros outside the matrix
bool encode_group_map(CUtensorMap *map, const void *A, int n, long long lda) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc) return false;
    cuuint64_t dims[2] = {(cuuint64_t)(2 * (long long)n), (cuuint64_t)n};
    cuuint64_t strides[1] = {(cuuint64_t)(2 * lda * 4)};
    cuuint32_t box[2] = {32, (cuuint32_t)kUmRows};
    cuuint32_t estr[2] = {1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void *>(A), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// BEM_GB300_TEST_WAIT_CYCLES: a bound (clock cycles) for the products'
// mbarrier waits in place of the default of about 2 s.  Only for tests that
// make a wait run out; read whenever a batch is set up.
// BEM_GB300_TEST_WAIT_KINDS: the product kinds the bound applies to (bit k:
// kind k; 0 Krylov products, 1 first refinement residuals, 2 residual
// updates); all by default.
int test_wait_kinds() {
    const char *v = std::getenv("BEM_GB300_TEST_WAIT_KINDS");
    return (v && *v) ? std::atoi(v) : 7;
}

long long test_wait_cycles() {
    const char *v = std::getenv("BEM_GB300_TEST_WAIT_CYCLES");
    if (!v || !*v) return 0;
    const long long c = std::atoll(v);
    return c > 0 ? c : 0;
}
}  // namespace

Engine::~Engine() {
    if (st_) cudaStreamSynchronize(st_);
    for (auto &x : exec_)
        if (x) cudaGraphExecDestroy(x);
    for (auto &e : ev_)
        if (e) cudaEventDestroy(e);
    cudaFree(d_tab_);
    cudaFree(d_st_);
    cudaFree(d_items_);
    if (h_tab_) cudaFreeHost(h_tab_);
    if (h_st_) cudaFreeHost(h_st_);
}

cudaError_t Engine::ensure_init() {
    if (d_tab_) return cudaSuccess;
    cudaError_t e = krylov_prepare();
    if (e == cudaSuccess) e = cudaMalloc(&d_tab_, sizeof(KTable));
    if (e == cudaSuccess) e = cudaMalloc(&d_st_, sizeof(KState) * kMaxSys);
    if (e == cudaSuccess) e = cudaMallocHost(&h_tab_, sizeof(KTable));
    if (e == cudaSuccess) e = cudaMallocHost(&h_st_, sizeof(KState) * kMaxSys);
    for (auto &ev : ev_)
        if (e == cudaSuccess) e = cudaEventCreate(&ev);
    if (e == cudaSuccess) {
        std::memset(h_tab_, 0, sizeof(KTable));
        std::memset(h_st_, 0, sizeof(KState) * kMaxSys);
        e = cudaMemcpyAsync(d_tab_, h_tab_, sizeof(KTable), cudaMemcpyHostToDevice, st_);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st_);
    return e;
}

cudaError_t Engine::set_batch(const std::vector<KSys> &sys, const std::vector<KState> &init) {
    if (sys.size() != init.size() || sys.size() > (size_t)kMaxSys) return cudaErrorInvalidValue;
    cudaError_t e = ensure_init();
    if (e != cudaSuccess) return e;
    // the previous replay (if any) has completed: run_body synchronizes
    const int B = (int)sys.size();
    items_.clear();
    int vb_total = 0;
    for (int b = 0; b < B; ++b) vb_total += sys[b].nvb;
    items_.reserve((size_t)vb_total);
    for (int b = 0; b < B; ++b)
        for (int q = 0; q < sys[b].nvb; ++q) items_.push_back(make_int2(b, q));
    if (items_.size() > items_cap_) {
        cudaFree(d_items_);
        d_items_ = nullptr;
        items_cap_ = 0;
        const size_t cap = items_.size() + items_.size() / 4 + 1024;
        e = cudaMalloc(&d_items_, cap * sizeof(int2));
        if (e != cudaSuccess) return e;
        items_cap_ = cap;
    }
    if (!items_.empty())
        e = cudaMemcpyAsync(d_items_, items_.data(), items_.size() * sizeof(int2), cudaMemcpyHostToDevice, st_);
    if (e != cudaSuccess) return e;
    std::memset(h_tab_, 0, sizeof(KTable));   // plans are rebuilt on the device below
    h_tab_->B = B;
    h_tab_->prec = prec_;
    h_tab_->vb_total = vb_total;
    h_tab_->vb_items = d_items_;
    h_tab_->wait_cycles = test_wait_cycles();
    h_tab_->wait_kinds = test_wait_kinds();
    for (int b = 0; b < B; ++b) {
        h_tab_->sys[b] = sys[b];
        h_tab_->sys[b].st = d_st_ + b;
        h_tab_->sys[b].shared = 0;
        h_tab_->pcw_any |= sys[b].pcw;
        h_st_[b] = init[b];
    }
    // complex64 systems next to each other on the same matrix (the right-hand
    // sides of one solver) form groups whose products share each read of A
    int ng = 0;
    for (int b = 0; b < B && prec_ == 1;) {
        int e = b + 1;
        while (e < B && e - b < kMaxGroup && sys[e].A == sys[b].A) ++e;
        if (e - b >= 2) {
            h_tab_->grp[ng].first = b;
            h_tab_->grp[ng].count = e - b;
            ++ng;
            for (int q = b; q < e; ++q) {
                h_tab_->sys[q].shared = 1;
                h_tab_->sys[q].nchunk = 1;   // the group product writes full rows
            }
        }
        b = e;
    }
    h_tab_->n_groups = ng;
    groups_ = ng;
    blr_ = 0;
    dense_ = 0;
    for (int b = 0; b < B; ++b) {
        if (h_tab_->sys[b].shared) continue;
        if (h_tab_->sys[b].blr_nb > 0) ++blr_;
        else ++dense_;
    }
    // the groups' Krylov products on the 5th-generation tensor cores need a
    // TMA map of each group's matrix; without them the warp-level kernel runs
    bool umma = ng > 0 && group_product_umma();
    for (int q = 0; q < ng && umma; ++q) {
        const KSys &g0 = h_tab_->sys[h_tab_->grp[q].first];
        umma = encode_group_map(&h_tab_->gmap[q], g0.A, g0.n, g0.lda);
    }
    h_tab_->grp_umma = umma ? 1 : 0;
    e = cudaMemcpyAsync(d_tab_, h_tab_, sizeof(KTable), cudaMemcpyHostToDevice, st_);
    if (e == cudaSuccess && B > 0)
        e = cudaMemcpyAsync(d_st_, h_st_, sizeof(KState) * B, cudaMemcpyHostToDevice, st_);
    // systems may be in the middle of a cycle: their next products need plans
    if (e == cudaSuccess) e = launch_plans(d_tab_, st_);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st_);
    B_ = B;
    mv_ms_ = 0.0;
    bodies_ = 0;
    return e;
}

cudaError_t Engine::time_product(const KSys &sys, float *ms) {
    cudaError_t e = ensure_init();
    if (e != cudaSuccess) return e;
    std::memset(h_tab_, 0, sizeof(KTable));
    h_tab_->B = 1;
    h_tab_->prec = prec_;
    h_tab_->vb_total = sys.nvb;
    h_tab_->wait_cycles = test_wait_cycles();
    h_tab_->wait_kinds = test_wait_kinds();
    h_tab_->sys[0] = sys;
    h_tab_->sys[0].st = d_st_;
    h_tab_->sys[0].shared = 0;
    const int strip = sys.strip > 0 ? sys.strip : kTmaStrip;
    KPlan &p = h_tab_->plan[0];
    p.n = 1;
    p.sys[0] = 0;
    p.off[0] = 0;
    p.off[1] = sys.A16 ? mv_items16(sys.n, strip) : mv_items_of(sys.n, prec_, strip);
    e = cudaMemcpyAsync(d_tab_, h_tab_, sizeof(KTable), cudaMemcpyHostToDevice, st_);
    float best = 1e30f;
    for (int rep = 0; rep < 3 && e == cudaSuccess; ++rep) {
        e = cudaEventRecord(ev_[0], st_);
        if (e == cudaSuccess) e = launch_product(d_tab_, prec_, st_);
        if (e == cudaSuccess) e = cudaEventRecord(ev_[1], st_);
        if (e == cudaSuccess) e = cudaEventSynchronize(ev_[1]);
        float t = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&t, ev_[0], ev_[1]);
        if (e == cudaSuccess && rep > 0 && t < best) best = t;
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h_tab_->err, &d_tab_->err, sizeof(int), cudaMemcpyDeviceToHost, st_);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st_);
    if (e == cudaSuccess && h_tab_->err) e = cudaErrorLaunchTimeout;
    count_launches(3);
    *ms = best;
    B_ = 0;   // the table no longer holds a batch
    return e;
}

cudaError_t Engine::run_body() {
    cudaError_t e = ensure_init();
    if (e != cudaSuccess) return e;
    const int v = (groups_ > 0 ? 1 : 0) | (blr_ > 0 ? 2 : 0) | (dense_ > 0 ? 4 : 0);
    if (!exec_[v]) {
        cudaGraph_t g = nullptr;
        e = cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return e;
        cudaError_t le = launch_krylov_body(prec_, d_tab_, ev_, st_, &body_launches_[v], (v & 1) != 0,
                                                   (v & 2) != 0, (v & 4) != 0);
        e = cudaStreamEndCapture(st_, &g);
        if (le != cudaSuccess) e = le;
        if (e == cudaSuccess) e = cudaGraphInstantiate(&exec_[v], g, 0);
        if (g) cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            exec_[v] = nullptr;
            return e;
        }
    }
    e = cudaGraphLaunch(exec_[v], st_);
    if (e == cudaSuccess && B_ > 0)
        e = cudaMemcpyAsync(h_st_, d_st_, sizeof(KState) * B_, cudaMemcpyDeviceToHost, st_);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h_tab_->err, &d_tab_->err, sizeof(int), cudaMemcpyDeviceToHost, st_);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st_);
    if (e != cudaSuccess) return e;
    if (h_tab_->err) return cudaErrorLaunchTimeout;   // a bounded wait in the product gave up
    count_launches(body_launches_[v]);
    ++bodies_;
    if (timing_ok_) {
        for (int q = 0; q <= kSteps; ++q) {
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, ev_[2 * q], ev_[2 * q + 1]) != cudaSuccess) {
                cudaGetLastError();
                timing_ok_ = false;
                break;
            }
            mv_ms_ += ms;
        }
    }
    return cudaSuccess;
}

}  // namespace bem
