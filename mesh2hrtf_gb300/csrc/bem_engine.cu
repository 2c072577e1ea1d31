// bem_engine.cu - host side of the batched Krylov engine: launch table,
// work-item lists, graph capture and replay.
#include <cuda_runtime.h>

#include <cstdlib>
#include <cstring>

#include "bem_engine.h"

namespace bem {

namespace {
// BEM_GB300_TEST_WAIT_CYCLES: a bound (clock cycles) for the products'
// mbarrier waits in place of the default of about 2 s.  Only for tests that
// make a wait run out; read whenever a batch is set up.
long long test_wait_cycles() {
    const char *v = std::getenv("BEM_GB300_TEST_WAIT_CYCLES");
    if (!v || !*v) return 0;
    const long long c = std::atoll(v);
    return c > 0 ? c : 0;
}
}  // namespace

Engine::~Engine() {
    if (st_) cudaStreamSynchronize(st_);
    if (exec_) cudaGraphExecDestroy(exec_);
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

cudaError_t Engine::run_body() {
    cudaError_t e = ensure_init();
    if (e != cudaSuccess) return e;
    if (!exec_) {
        cudaGraph_t g = nullptr;
        e = cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return e;
        cudaError_t le = launch_krylov_body(prec_, d_tab_, ev_, st_, &body_launches_);
        e = cudaStreamEndCapture(st_, &g);
        if (le != cudaSuccess) e = le;
        if (e == cudaSuccess) e = cudaGraphInstantiate(&exec_, g, 0);
        if (g) cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            exec_ = nullptr;
            return e;
        }
    }
    e = cudaGraphLaunch(exec_, st_);
    if (e == cudaSuccess && B_ > 0)
        e = cudaMemcpyAsync(h_st_, d_st_, sizeof(KState) * B_, cudaMemcpyDeviceToHost, st_);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h_tab_->err, &d_tab_->err, sizeof(int), cudaMemcpyDeviceToHost, st_);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st_);
    if (e != cudaSuccess) return e;
    if (h_tab_->err) return cudaErrorLaunchTimeout;   // a bounded wait in the product gave up
    count_launches(body_launches_);
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
