// bem_engine.h - host side of the batched Krylov engine (bem_gmres.cu).
//
// An Engine owns a device launch table (KTable), the systems' GMRES states,
// the work-item lists of the kernels, and one CUDA graph of the iteration
// body, captured at the first replay.  The table and states live in device
// memory, so the graph stays valid while systems come and go: set_batch()
// rewrites them between replays.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "bem_internal.h"

namespace bem {

// Device work queues and kernel grids; call once per device before capture.
cudaError_t krylov_prepare();

class Engine {
public:
    Engine(int prec, cudaStream_t st) : prec_(prec), st_(st) {}
    ~Engine();
    Engine(const Engine &) = delete;
    Engine &operator=(const Engine &) = delete;

    // Replaces the batch with sys[0..B) and their states (KSys::st is set here).
    cudaError_t set_batch(const std::vector<KSys> &sys, const std::vector<KState> &init);
    // One replay of the iteration body; afterwards states() holds the
    // systems' states as of the end of that body.
    cudaError_t run_body();
    const KState *states() const { return h_st_; }
    int size() const { return B_; }
    int precision() const { return prec_; }
    cudaStream_t stream() const { return st_; }
    // Time (ms, best of two launches after one warm-up) of one Krylov product
    // of a complex64 system alone, with the strip height in sys.strip; for
    // the tuner, before set_batch (it overwrites the launch table).
    cudaError_t time_product(const KSys &sys, float *ms);
    // device time of the matrix-vector products (ms) and body replays since set_batch
    double matvec_ms() const { return mv_ms_; }
    long long bodies() const { return bodies_; }
    bool timing_ok() const { return timing_ok_; }

private:
    cudaError_t ensure_init();
    int prec_;
    cudaStream_t st_;
    int B_ = 0;
    KTable *d_tab_ = nullptr, *h_tab_ = nullptr;
    KState *d_st_ = nullptr, *h_st_ = nullptr;
    int2 *d_items_ = nullptr;
    size_t items_cap_ = 0;
    std::vector<int2> items_;
    // the iteration body's variants: with the shared-matrix (group) products
    // (bit 0), with the block low-rank product (bit 1), with the product of
    // single systems from A or its fp16 copy (bit 2); each captured at its
    // first replay
    cudaGraphExec_t exec_[8] = {};
    int body_launches_[8] = {};
    int groups_ = 0;   // shared-matrix groups of the current batch
    int blr_ = 0;      // systems of the current batch with a block low-rank copy
    int dense_ = 0;    // single systems whose Krylov products read A or its fp16 copy
    cudaEvent_t ev_[2 * (kSteps + 1)] = {};
    double mv_ms_ = 0.0;
    long long bodies_ = 0;
    bool timing_ok_ = true;
};

}  // namespace bem
