// bem_gmres.cu - restarted GMRES with iterative refinement for a batch of
// dense BEM systems, driven entirely on the device.
//
// Counterpart of NumCalc's NC_IterativeSolverCGS with its preconditioners
// and matrix-vector product (NC_CommonFunctions.cpp:1066-1245, 1322-1721).
// The method is different (GMRES with a block-Jacobi preconditioner, its
// window correction and refinement instead of CGS with a threshold ILU); the
// system solved and the stopping rule (relative residual below 1e-9 by
// default) are NumCalc's.
//
// Every system of the batch carries a small state machine (KState) in device
// memory.  An iteration body runs kSteps Arnoldi steps for each system in
// phase ARNOLDI and then the end of cycle for each system in phase UPDATE;
// kernels skip the systems that are in another phase.  The body never needs
// the host, so it is captured once as a CUDA graph and replayed; the host
// reads the states after each replay and admits or retires systems between
// replays.  The per-system arithmetic does not depend on the other systems of
// the batch, so a system's result is the same alone and in any mix.
//
// Arnoldi step k (8 launches):
//   k_mv_tma      w_parts = A z_k               complex64: bulk-copy pipeline
//   (k_mv64)                                    complex128: persistent tiles
//   k_dot1        w = sum parts; h1 = V^H w     per 256-row block
//   k_axpy<1>     w -= V h1; h2 = V^H w         (classical Gram-Schmidt, twice)
//   k_axpy<2>     w -= V h2; |w|^2 partials
//                 (a system flagged cgs1 takes one pass: k_axpy<1> passes
//                 it by and k_axpy<2> subtracts V h1)
//   k_scale       v_{k+1} = w / |w|; z_{k+1} = M^{-1} v_{k+1}
//   k_pcwin,      the preconditioner's window correction:
//   k_pcfin       M^{-1} = X (2 I - A_w X), X block-Jacobi (2 launches)
//   k_givens      column k of H, rotations, residual estimate, phase
// End of cycle (8 launches):
//   k_trisolve    y = H^{-1} g                   warp per system
//   k_xupdate     x += M^{-1} (V y)              (+ k_pcwin, k_pcfin)
//   k_mv_tma      b - A x with error-free products (the refinement residual)
//   k_resid       r, |r|^2 partials
//   k_decide      convergence / stagnation / limit, restart set-up
//   k_scale       v_0 = r / |r|; z_0 = M^{-1} v_0 (restarted systems)
//                 (+ k_pcwin, k_pcfin)
//
// Inner products are summed in a fixed order (per block, then over blocks in
// block order, every block computing the same sums), so results are
// deterministic run to run.
//
// complex128 systems run the Arnoldi vectors in FP64.  complex64 systems
// keep w and the basis V in float pairs with FP32 products and sums (GMRES
// in working precision inside the refinement, whose residuals stay FP64):
// an inner cycle needs three to five digits, and GB300's narrow FP64 pipe
// bounded the FP64 inner products and updates of these kernels.  H, the
// rotations and x stay FP64.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <atomic>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "bem_engine.h"
#include "bem_internal.h"
#include "bem_umma.h"

namespace bem {
namespace {

constexpr int kThreads = kVecBlock;        // vector kernels: one row per thread
constexpr int kMaxV = kMaxRestart + 1;     // basis vectors
static_assert(kThreads == 2 * kBlock, "a vector block holds two preconditioner blocks");
static_assert(kMaxV <= 64, "inner products are computed in groups of 8 up to 64 vectors");

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// error-free transformations (Knuth two-sum, FMA two-product)
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// FP64 row partial from a float-float pair; out of line so that the
// conversions are not executed (predicated) on the float-partial path.
__device__ __noinline__ void store_partial_f64(double2 *p, float4 o) {
    *p = make_double2((double)o.x + (double)o.y, (double)o.z + (double)o.w);
}

// Warp sums in FP32.  GB300's FP64 pipe is narrow (a warp instruction
// occupies it for many cycles), so the products reduce their row sums in
// FP32 and convert once per row; the butterfly leaves the same value on every
// lane (a + b == b + a).
__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
// Float-float pairs (s, e): two-sum at every level, about twice-FP32 accurate.
__device__ __forceinline__ void warp_sum_ff(float &s, float &e) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float s2 = __shfl_xor_sync(0xffffffffu, s, o), e2 = __shfl_xor_sync(0xffffffffu, e, o);
        float t, u;
        two_sum(s, s2, t, u);
        s = t;
        e = (e + e2) + u;
    }
}
__device__ __forceinline__ void acc_exact(float &s, float &e, float a, float b) {
    const float p = a * b;
    const float q = fmaf(a, b, -p);
    float t, u;
    two_sum(s, p, t, u);
    s = t;
    e += u + q;
}

// Does a system take part in a product of this kind?  0: Krylov product;
// 1: residual with error-free products (the first cycle's, and every one for
// complex128); 2: recursive residual update (complex64, later cycles).
__device__ __forceinline__ bool mv_active(const KState *st, int kind, int prec) {
    if (kind == 0) return st->phase == kPhaseArnoldi;
    if (st->phase != kPhaseUpdate || st->cycles == 0) return false;
    if (kind == 1) return prec == 0 || st->cycles == 1;
    return prec == 1 && st->cycles >= 2;
}

// ------------------------------------------------------------ launch plans
// Slot j of a plan with plan.off[j] <= item < plan.off[j + 1].
__device__ __forceinline__ int plan_find(const int *off, int n, int item) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (off[mid] <= item) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Copy of a plan in shared memory, loaded by the whole block.
struct PlanSmem {
    int n;
    int off[kMaxSys + 1];
    int sys[kMaxSys];
};
__device__ __forceinline__ void plan_load(const KPlan &p, PlanSmem &s) {
    if (threadIdx.x == 0) s.n = p.n;
    for (int i = threadIdx.x; i <= kMaxSys; i += blockDim.x) s.off[i] = p.off[i];
    for (int i = threadIdx.x; i < kMaxSys; i += blockDim.x) s.sys[i] = p.sys[i];
    __syncthreads();
}

// Rebuild plan `which` (a product kind, see mv_active) from the current
// phases; one block of kMaxSys threads, thread t = slot t.
__device__ void plan_build(KTable *tb, int which) {
    __shared__ int cnt[kMaxSys], act[kMaxSys];
    __shared__ unsigned gm[kMaxSys];
    const int t = threadIdx.x;
    int c = 0, cb = 0;
    if (t < tb->B) {
        const KSys &S = tb->sys[t];
        if (!S.shared && mv_active(S.st, which, tb->prec)) {
            const int strip = S.strip > 0 ? S.strip : kTmaStrip;
            if (which == 0 && S.blr_nb > 0) cb = S.blr_nb * S.nchunk;   // block low-rank copy
            else c = (which == 0 && S.A16) ? mv_items16(S.n, strip) : mv_items_of(S.n, tb->prec, strip);
        }
    }
    cnt[t] = c;
    act[t] = c > 0;
    // shared-matrix groups: members taking part, strips of the group
    unsigned mask = 0;
    if (t < tb->n_groups) {
        const KGroup g = tb->grp[t];
        for (int q = 0; q < g.count; ++q)
            if (mv_active(tb->sys[g.first + q].st, which, tb->prec)) mask |= 1u << q;
    }
    gm[t] = mask;
    __syncthreads();
    // exclusive prefix sums over the kMaxSys slots (warp scans, then the
    // warps' totals in order): the plan entries in slot order
    __shared__ int wsum[kMaxSys / 32][6];
    const int lane = t & 31, wp = t >> 5;
    const int ga = gm[t] ? 1 : 0;
    const int grows = which == 1 ? kGrpRowsExact : (which == 0 && tb->grp_umma ? kUmRows : kGrpRowsInner);
    const int gc = ga ? ceil_div(tb->sys[tb->grp[t].first].n, grows) : 0;
    const int ba = cb > 0 ? 1 : 0;
    int v[6] = {act[t], cnt[t], ga, gc, ba, cb};
#pragma unroll
    for (int q = 0; q < 6; ++q) {
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, v[q], o);
            if (lane >= o) v[q] += y;
        }
        if (lane == 31) wsum[wp][q] = v[q];
    }
    __syncthreads();
    int base[6] = {0, 0, 0, 0, 0, 0};
    for (int w = 0; w < wp; ++w)
#pragma unroll
        for (int q = 0; q < 6; ++q) base[q] += wsum[w][q];
    const int pos = base[0] + v[0] - act[t], off = base[1] + v[1] - cnt[t];
    const int gpos = base[2] + v[2] - ga, goff = base[3] + v[3] - gc;
    const int bpos = base[4] + v[4] - ba, boff = base[5] + v[5] - cb;
    KPlan &p = tb->plan[which];
    KPlan &gp = tb->gplan[which];
    if (act[t]) {
        p.sys[pos] = t;
        p.off[pos] = off;
    }
    if (ga) {
        gp.sys[gpos] = t;
        gp.off[gpos] = goff;
        tb->gmask[which][gpos] = gm[t];
    }
    if (which == 0 && ba) {
        tb->bplan.sys[bpos] = t;
        tb->bplan.off[bpos] = boff;
    }
    if (t == kMaxSys - 1) {
        p.n = base[0] + v[0];
        p.off[p.n] = base[1] + v[1];
        gp.n = base[2] + v[2];
        gp.off[gp.n] = base[3] + v[3];
        if (which == 0) {
            tb->bplan.n = base[4] + v[4];
            tb->bplan.off[tb->bplan.n] = base[5] + v[5];
        }
    }
    __syncthreads();
}

// ------------------------------------------------------------ matvec (complex128)
// Persistent grid; blocks take tiles (system, 32 rows x 1024 columns) from a
// queue.  The x chunk is staged in shared memory; 8 warps x 4 rows; each lane
// streams 16-byte loads (one complex128 entry) of its 4 rows.  The FP64 path
// is bound by the FP64 pipe (4 DFMA per entry), not by HBM.  The tile writes
// one partial per row; the consumer sums the chunks in order.
template <bool EXACT>
__global__ void __launch_bounds__(256, 4) k_mv64(KTable *tb, int kind) {
    __shared__ __align__(16) double2 xd[kMvChunk];
    __shared__ int item_s;
    __shared__ PlanSmem pl;
    plan_load(tb->plan[kind], pl);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int total = pl.off[pl.n];
    while (total > 0) {
        if (threadIdx.x == 0) item_s = (int)atomicAdd(&tb->mv_ctr[0], 1u);
        __syncthreads();
        const int item = item_s;
        __syncthreads();
        if (item >= total) break;
        const int j = plan_find(pl.off, pl.n, item);
        const KSys &S = tb->sys[pl.sys[j]];
        const KState *st = S.st;
        const int local = item - pl.off[j];
        const int n = S.n;
        const int chunk = local % S.nchunk, tile = local / S.nchunk;
        const int c0 = chunk * kMvChunk, len = min(kMvChunk, n - c0);
        const double2 *xs = EXACT ? S.x : (S.pc ? S.z : S.V + (size_t)st->k * S.ldv);
        for (int t = threadIdx.x; t < len; t += blockDim.x) xd[t] = xs[c0 + t];
        __syncthreads();
        const int row0 = tile * kMvRows + warp * 4;
        double re[4] = {0.0, 0.0, 0.0, 0.0}, im[4] = {0.0, 0.0, 0.0, 0.0};
        const double2 *A = (const double2 *)S.A;
#pragma unroll 2
        for (int c = lane; c < len; c += 32) {
            const double2 xv = xd[c];
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                if (row0 + r < n) {
                    const double2 a = __ldcs(A + (size_t)(row0 + r) * S.lda + c0 + c);
                    re[r] = fma(a.x, xv.x, re[r]);
                    re[r] = fma(-a.y, xv.y, re[r]);
                    im[r] = fma(a.x, xv.y, im[r]);
                    im[r] = fma(a.y, xv.x, im[r]);
                }
            }
        }
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            re[r] = warp_sum_d(re[r]);
            im[r] = warp_sum_d(im[r]);
        }
        if (lane == 0)
#pragma unroll
            for (int r = 0; r < 4; ++r)
                if (row0 + r < n) S.mvp[(size_t)chunk * n + row0 + r] = make_double2(re[r], im[r]);
    }
    // the last block to leave resets the queue for the next launch
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&tb->mv_ctr[1], 1u) == gridDim.x - 1) {
            tb->mv_ctr[0] = 0u;
            tb->mv_ctr[1] = 0u;
            __threadfence();
        }
    }
}

// ------------------------------------------------------------ bulk-copy matvec
// complex64 product with a bulk-copy (TMA) pipeline.  A persistent block per
// SM: one producer warp and 8 consumer warps.  The producer takes items
// (system, 1024-column chunk, strip of 64 rows) from the queue and streams
// them through a ring of kTmaStages stages of kTmaRows row segments (8 KB
// each, one cp.async.bulk per segment) into shared memory; the chunk of x
// (float hi parts, or hi/lo pairs for the refinement residual) goes into one
// of two x buffers.  mbarriers carry the byte counts (full) and the
// consumers' releases (empty).  Consumer warp w < 8 takes row w of a stage.
// Krylov products of systems with an fp16 copy of A (KSys::A16) stream that
// copy instead, with items of two column chunks so that row segments stay
// 8 KB (the number of bulk copies an SM completes per second, not their
// size, limits 4 KB segments); consumer warp w takes row w & 7 over chunk
// w >> 3 of the item and scales its sum by the row's power-of-two scale.
// Every wait is bounded (kWaitCycles); on expiry the kernel sets tb->err,
// lets its own copies land and returns.
constexpr int kTmaStages = 3;
constexpr int kTmaConsumers = 16;
static_assert(kTmaConsumers == 2 * kTmaRows, "one consumer warp per (row, chunk) of an fp16 stage");
constexpr long long kWaitCycles = 4000000000LL;   // about 2 s at 2 GHz
constexpr int kStageBytes = kTmaRows * kMvChunk * 8;   // 64 KB

struct TmaMeta {
    int b, chunk, row0, nrows, len, first, last, xslot, h;
};
static_assert(kTmaRows * 2 * kMvChunk * 4 == kStageBytes, "an fp16 stage (two chunks) fills the stage buffer");

__device__ __forceinline__ float2 h2f(unsigned u) {
    __half2 h;
    *reinterpret_cast<unsigned *>(&h) = u;
    return __half22float2(h);
}

// x buffers: hi/lo pairs of one chunk (refinement residual) or hi parts of
// two chunks (fp16 Krylov items)
__host__ __device__ constexpr int tma_x_bytes(bool) { return kMvChunk * 16; }
__host__ __device__ constexpr int tma_smem_bytes(bool exact) {
    return kTmaStages * kStageBytes + 2 * tma_x_bytes(exact) + 256;
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint32_t a, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t a, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t a) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(a) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t a, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    return ok != 0;
}
// non-blocking test of the same
__device__ __forceinline__ bool mbar_test(uint32_t a, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait for the completion of the phase with the given parity; lim
// is the bound in clock cycles.  try_wait may suspend the thread for a
// system-dependent time before it reports an incomplete phase, so a bound
// shorter than the default (set by a test that makes a wait run out) polls
// with the non-blocking test instead.
__device__ __forceinline__ bool mbar_wait(uint32_t a, uint32_t parity, int *err, long long lim = kWaitCycles) {
    if (lim < kWaitCycles) {
        const long long t0 = clock64();
        while (!mbar_test(a, parity)) {
            if (clock64() - t0 > lim) {
                atomicExch(err, 1);
                return false;
            }
        }
        return true;
    }
    if (mbar_try(a, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try(a, parity)) {
        if (clock64() - t0 > lim) {
            atomicExch(err, 1);
            return false;
        }
    }
    return true;
}
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t mbar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(mbar)
                 : "memory");
}

template <bool EXACT>
__global__ void __launch_bounds__(32 * (kTmaConsumers + 1), 1) k_mv_tma(KTable *tb, int kind) {
    extern __shared__ __align__(128) unsigned char smem[];
    unsigned char *ring = smem;                                       // kTmaStages x 64 KB
    unsigned char *xbuf = smem + kTmaStages * kStageBytes;           // 2 x chunk of x
    uint64_t *bars = reinterpret_cast<uint64_t *>(xbuf + 2 * tma_x_bytes(EXACT));
    // bars: full[3], empty[3], xfull[2], xempty[2]; then the stage metadata
    TmaMeta *meta = reinterpret_cast<TmaMeta *>(bars + 2 * kTmaStages + 4);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + kTmaStages);
    const uint32_t xfull0 = smem_u32(bars + 2 * kTmaStages), xempty0 = smem_u32(bars + 2 * kTmaStages + 2);
    if (threadIdx.x == 0) {
        for (int s = 0; s < kTmaStages; ++s) {
            mbar_init(full0 + 8 * s, 1);
            mbar_init(empty0 + 8 * s, kTmaConsumers);
        }
        for (int q = 0; q < 2; ++q) {
            mbar_init(xfull0 + 8 * q, 1);
            mbar_init(xempty0 + 8 * q, kTmaConsumers);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __shared__ PlanSmem pl;
    plan_load(tb->plan[kind], pl);   // includes a block barrier
    int *err = &tb->err;
    // bound of the waits (the drains of in-flight copies keep the full bound)
    const long long lim = (tb->wait_cycles > 0 && ((tb->wait_kinds >> kind) & 1)) ? tb->wait_cycles : kWaitCycles;
    if (warp == kTmaConsumers) {
        // ---------------- producer warp: lane 0 takes the items and keeps the
        // barriers, lane r issues the bulk copy of row r of a stage (one
        // thread issuing every copy caps the copy rate below HBM speed for
        // the 4 KB fp16 segments)
        const unsigned kAll = 0xffffffffu;
        const int total = pl.off[pl.n];
        int stage = 0, xs = 0;
        uint32_t eph = 1, xeph[2] = {1, 1};   // a fresh barrier's previous phase counts as complete
        int issued[kTmaStages] = {0, 0, 0};   // stage holds copies not yet seen complete by us
        uint32_t fph[kTmaStages] = {0, 0, 0};
        int xiss[2] = {0, 0};                 // the same for the two x buffers
        uint32_t xfp[2] = {0, 0};
        bool ok = true;
        while (ok && total > 0) {
            int item = 0;
            if (lane == 0) item = (int)atomicAdd(&tb->mv_ctr[0], 1u);
            item = __shfl_sync(kAll, item, 0);
            if (item >= total) break;
            const int j = plan_find(pl.off, pl.n, item);
            const int sb = pl.sys[j], local = item - pl.off[j];
            const KSys &S = tb->sys[sb];
            const int n = S.n;
            const bool h = !EXACT && kind == 0 && S.A16 != nullptr;   // fp16 copy of A
            const int span = h ? 2 * kMvChunk : kMvChunk;              // columns per item
            const int nblk = h ? (S.nchunk + 1) / 2 : S.nchunk;
            const int blk = local % nblk, strip = local / nblk;
            const int chunk = h ? 2 * blk : blk;                       // first chunk of the item
            const int c0 = blk * span, len = min(span, n - c0), lenp = (len + 1) & ~1;
            const int sh = S.strip > 0 ? S.strip : kTmaStrip;   // rows per item
            const int rbase = strip * sh;
            const int rps = kTmaRows;
            const int nst = min(sh / rps, (n - rbase + rps - 1) / rps);
            // bytes per row segment: fp16 copies move whole 16-byte groups of 4 entries
            const uint32_t seg = h ? (uint32_t)(((len + 3) & ~3) * 4) : (uint32_t)(lenp * 8);
            const uint32_t pitch = kMvChunk * 8;
            const size_t lda = (size_t)S.lda;
            const unsigned char *abase = h ? (const unsigned char *)S.A16 : (const unsigned char *)S.A;
            const size_t esz = h ? 4 : 8;
            // x chunk
            int w = 1;
            if (lane == 0) w = mbar_wait(xempty0 + 8 * xs, xeph[xs], err, lim);
            if (!__shfl_sync(kAll, w, 0)) { ok = false; break; }
            xeph[xs] ^= 1;
            if (lane == 0) {
                const uint32_t xdst = smem_u32(xbuf + xs * tma_x_bytes(EXACT));
                if (EXACT) {
                    mbar_expect_tx(xfull0 + 8 * xs, kMvChunk * 16);
                    bulk_g2s(xdst, S.xf + c0, kMvChunk * 16, xfull0 + 8 * xs);
                } else {
                    mbar_expect_tx(xfull0 + 8 * xs, lenp * 8);
                    bulk_g2s(xdst, S.xh + c0, lenp * 8, xfull0 + 8 * xs);
                }
            }
            xiss[xs] = 1;
            xfp[xs] ^= 1;
            for (int g = 0; g < nst; ++g) {
                if (lane == 0) w = mbar_wait(empty0 + 8 * stage, eph, err, lim);
                if (!__shfl_sync(kAll, w, 0)) { ok = false; break; }
                const int row0 = rbase + g * rps, nrows = min(rps, n - row0);
                if (lane == 0) {
                    TmaMeta mt;
                    mt.b = sb; mt.chunk = chunk; mt.row0 = row0; mt.nrows = nrows; mt.len = len;
                    mt.first = g == 0; mt.last = g == nst - 1; mt.xslot = xs; mt.h = h;
                    meta[stage] = mt;
                    mbar_expect_tx(full0 + 8 * stage, (uint32_t)nrows * seg);
                }
                __syncwarp();
                if (lane < nrows)
                    bulk_g2s(smem_u32(ring + stage * kStageBytes) + lane * pitch,
                             abase + ((size_t)(row0 + lane) * lda + c0) * esz, seg, full0 + 8 * stage);
                issued[stage] = 1;
                fph[stage] ^= 1;
                if (++stage == kTmaStages) { stage = 0; eph ^= 1; }
            }
            xs ^= 1;
        }
        if (lane == 0) {
            if (ok) {
                // sentinel: consumers stop at the next stage
                if (mbar_wait(empty0 + 8 * stage, eph, err, lim)) {
                    meta[stage].b = -1;
                    mbar_arrive(full0 + 8 * stage);
                } else {
                    ok = false;
                }
            }
            if (!ok) {
                // a wait gave up: let this block's copies (stages and x
                // buffers) land before leaving
                for (int s = 0; s < kTmaStages; ++s)
                    if (issued[s]) mbar_wait(full0 + 8 * s, fph[s] ^ 1, err);
                for (int q = 0; q < 2; ++q)
                    if (xiss[q]) mbar_wait(xfull0 + 8 * q, xfp[q] ^ 1, err);
            }
            __threadfence();
            if (atomicAdd(&tb->mv_ctr[1], 1u) == gridDim.x - 1) {
                tb->mv_ctr[0] = 0u;
                tb->mv_ctr[1] = 0u;
                __threadfence();
            }
        }
        return;
    }
    // ---------------- consumers: warp w takes row w of each stage
    int stage = 0;
    uint32_t fph = 0, xph[2] = {0, 0};
    while (true) {
        if (!mbar_wait(full0 + 8 * stage, fph, err, lim)) return;
        const TmaMeta mt = meta[stage];
        if (mt.b < 0) return;
        const KSys &S = tb->sys[mt.b];
        if (mt.first) {
            if (!mbar_wait(xfull0 + 8 * mt.xslot, xph[mt.xslot], err, lim)) return;
        }
        const unsigned char *xb = xbuf + mt.xslot * tma_x_bytes(EXACT);
        // this warp's row sum as float-float (hi, lo) pairs of the real and
        // imaginary parts, written after the stage is released
        float4 o0 = make_float4(0.f, 0.f, 0.f, 0.f);
        int nout = 0;
        float sca = 1.f;
        bool released = false;   // stage handed back before the arithmetic
        if (!EXACT && mt.h) {
            // fp16: row w & 7 over the item's chunk w >> 3.  The warp copies its
            // 4 KB of A into registers and releases the stage at once, so the
            // slot refills while it computes; two accumulators per component
            // (even / odd entries) shorten the dependency chains.
            const int r = warp & (kTmaRows - 1), half = warp >> 3;
            const int len = mt.len - half * kMvChunk;   // columns of this chunk
            const bool act = r < mt.nrows && len > 0;
            const int len2 = act ? min(len, kMvChunk) >> 1 : 0;
            const uint2 *Aa = reinterpret_cast<const uint2 *>(ring + stage * kStageBytes + r * kMvChunk * 8 +
                                                              half * kMvChunk * 4);
            const bool full = len2 == kMvChunk / 2;   // whole chunk: no guards
            uint2 av[kMvChunk / 64];
            if (full) {
#pragma unroll
                for (int q = 0; q < kMvChunk / 64; ++q) av[q] = Aa[lane + 32 * q];
            } else {
#pragma unroll
                for (int q = 0; q < kMvChunk / 64; ++q) {
                    const int c = lane + 32 * q;
                    av[q] = c < len2 ? Aa[c] : make_uint2(0u, 0u);
                }
            }
            unsigned atail = 0u;
            const bool tail = act && len < kMvChunk && (len & 1);
            if (tail && lane == 0) atail = reinterpret_cast<const unsigned *>(Aa)[len - 1];
            // every lane's loads have returned before the warp passes the
            // barrier (the value below needs them), so the slot may be refilled
            unsigned dep = atail;
#pragma unroll
            for (int q = 0; q < kMvChunk / 64; ++q) dep |= av[q].x | av[q].y;
            asm volatile("" ::"r"(dep));
            __syncwarp();
            if (lane == 0) mbar_arrive(empty0 + 8 * stage);
            released = true;
            if (act) {
                sca = S.rs[(size_t)(mt.row0 + r) * mv_chunks(S.n) + mt.chunk + half];
                const float4 *x4 = reinterpret_cast<const float4 *>(xb + half * kMvChunk * 8);
                float ar = 0.f, ai = 0.f, br = 0.f, bi = 0.f;
                if (full) {
#pragma unroll
                    for (int q = 0; q < kMvChunk / 64; ++q) {
                        const float4 xv = x4[lane + 32 * q];
                        const float2 a0 = h2f(av[q].x), a1 = h2f(av[q].y);
                        ar = fmaf(a0.x, xv.x, ar); ar = fmaf(-a0.y, xv.y, ar);
                        ai = fmaf(a0.x, xv.y, ai); ai = fmaf(a0.y, xv.x, ai);
                        br = fmaf(a1.x, xv.z, br); br = fmaf(-a1.y, xv.w, br);
                        bi = fmaf(a1.x, xv.w, bi); bi = fmaf(a1.y, xv.z, bi);
                    }
                } else {
#pragma unroll
                    for (int q = 0; q < kMvChunk / 64; ++q) {
                        const int c = lane + 32 * q;
                        if (c < len2) {
                            const float4 xv = x4[c];
                            const float2 a0 = h2f(av[q].x), a1 = h2f(av[q].y);
                            ar = fmaf(a0.x, xv.x, ar); ar = fmaf(-a0.y, xv.y, ar);
                            ai = fmaf(a0.x, xv.y, ai); ai = fmaf(a0.y, xv.x, ai);
                            br = fmaf(a1.x, xv.z, br); br = fmaf(-a1.y, xv.w, br);
                            bi = fmaf(a1.x, xv.w, bi); bi = fmaf(a1.y, xv.z, bi);
                        }
                    }
                }
                if (tail && lane == 0) {
                    const float2 xv = reinterpret_cast<const float2 *>(x4)[len - 1];
                    const float2 at = h2f(atail);
                    ar = fmaf(at.x, xv.x, ar); ar = fmaf(-at.y, xv.y, ar);
                    ai = fmaf(at.x, xv.y, ai); ai = fmaf(at.y, xv.x, ai);
                }
                // power-of-two segment scale: exact in float
                o0 = make_float4(warp_sum_f(ar + br) * sca, 0.f, warp_sum_f(ai + bi) * sca, 0.f);
                nout = 1;
            }
        } else if (warp < mt.nrows) {
            const float4 *A4 = reinterpret_cast<const float4 *>(ring + stage * kStageBytes) + warp * (kMvChunk / 2);
            const int len = mt.len, len2 = len >> 1;
            float sr = 0.f, si = 0.f, er = 0.f, ei = 0.f;
            if (!EXACT) {
                const float4 *x4 = reinterpret_cast<const float4 *>(xb);   // hi parts of entries 2c, 2c + 1
#pragma unroll 4
                for (int c = lane; c < len2; c += 32) {
                    const float4 a = A4[c], xv = x4[c];
                    sr = fmaf(a.x, xv.x, sr); sr = fmaf(-a.y, xv.y, sr);
                    si = fmaf(a.x, xv.y, si); si = fmaf(a.y, xv.x, si);
                    sr = fmaf(a.z, xv.z, sr); sr = fmaf(-a.w, xv.w, sr);
                    si = fmaf(a.z, xv.w, si); si = fmaf(a.w, xv.z, si);
                }
                if ((len & 1) && lane == 0) {
                    const float2 a = reinterpret_cast<const float2 *>(A4)[len - 1];
                    const float2 xv = reinterpret_cast<const float2 *>(xb)[len - 1];
                    sr = fmaf(a.x, xv.x, sr); sr = fmaf(-a.y, xv.y, sr);
                    si = fmaf(a.x, xv.y, si); si = fmaf(a.y, xv.x, si);
                }
            } else {
                // x chunk permuted: entry 2c at xa[c], entry 2c + 1 at xb2[c].
                // Even and odd entries, and the two terms of each component,
                // accumulate into separate float-float pairs (one exact
                // product per pair and iteration), merged below.
                const float4 *xa = reinterpret_cast<const float4 *>(xb), *xb2 = xa + kMvChunk / 2;
                float sr2 = 0.f, si2 = 0.f, er2 = 0.f, ei2 = 0.f;   // odd entries
                float sr3 = 0.f, si3 = 0.f, er3 = 0.f, ei3 = 0.f;   // second terms, even
                float sr4 = 0.f, si4 = 0.f, er4 = 0.f, ei4 = 0.f;   // second terms, odd
#pragma unroll 2
                for (int c = lane; c < len2; c += 32) {
                    const float4 a = A4[c], x0 = xa[c], x1 = xb2[c];
                    acc_exact(sr, er, a.x, x0.x); acc_exact(sr3, er3, -a.y, x0.y);
                    acc_exact(si, ei, a.x, x0.y); acc_exact(si3, ei3, a.y, x0.x);
                    er = fmaf(a.x, x0.z, er); er3 = fmaf(-a.y, x0.w, er3);
                    ei = fmaf(a.x, x0.w, ei); ei3 = fmaf(a.y, x0.z, ei3);
                    acc_exact(sr2, er2, a.z, x1.x); acc_exact(sr4, er4, -a.w, x1.y);
                    acc_exact(si2, ei2, a.z, x1.y); acc_exact(si4, ei4, a.w, x1.x);
                    er2 = fmaf(a.z, x1.z, er2); er4 = fmaf(-a.w, x1.w, er4);
                    ei2 = fmaf(a.z, x1.w, ei2); ei4 = fmaf(a.w, x1.z, ei4);
                }
                {
                    float t, u;
                    two_sum(sr, sr3, t, u); sr = t; er += er3 + u;
                    two_sum(si, si3, t, u); si = t; ei += ei3 + u;
                    two_sum(sr2, sr4, t, u); sr2 = t; er2 += er4 + u;
                    two_sum(si2, si4, t, u); si2 = t; ei2 += ei4 + u;
                    two_sum(sr, sr2, t, u); sr = t; er += er2 + u;
                    two_sum(si, si2, t, u); si = t; ei += ei2 + u;
                }
                if ((len & 1) && lane == 0) {
                    const float2 a = reinterpret_cast<const float2 *>(A4)[len - 1];
                    const float4 x0 = xa[(len - 1) >> 1];
                    acc_exact(sr, er, a.x, x0.x); acc_exact(sr, er, -a.y, x0.y);
                    acc_exact(si, ei, a.x, x0.y); acc_exact(si, ei, a.y, x0.x);
                    er = fmaf(a.x, x0.z, er); er = fmaf(-a.y, x0.w, er);
                    ei = fmaf(a.x, x0.w, ei); ei = fmaf(a.y, x0.z, ei);
                }
            }
            if (EXACT) {
                warp_sum_ff(sr, er);
                warp_sum_ff(si, ei);
                o0 = make_float4(sr, er, si, ei);
            } else {
                o0 = make_float4(warp_sum_f(sr), 0.f, warp_sum_f(si), 0.f);
            }
            nout = 1;
        }
        __syncwarp();
        if (lane == 0) {
            if (!released) mbar_arrive(empty0 + 8 * stage);
            if (mt.last) mbar_arrive(xempty0 + 8 * mt.xslot);
            // row partial of chunk (w >> 3 for fp16 items), row w (& 7): float for
            // the Krylov products (summed in FP32 by k_dot1), FP64 for the
            // residuals (summed in FP64 by k_resid)
            const size_t o = (size_t)mt.chunk * S.n + mt.row0 +
                             ((!EXACT && mt.h) ? (size_t)(warp >> 3) * S.n + (warp & (kTmaRows - 1)) : (size_t)warp);
            if (nout > 0) {
                if (!EXACT && kind == 0)
                    reinterpret_cast<float2 *>(S.mvp)[o] = make_float2(o0.x + o0.y, o0.z + o0.w);
                else
                    store_partial_f64(S.mvp + o, o0);
            }
        }
        if (mt.first) xph[mt.xslot] ^= 1;
        if (++stage == kTmaStages) { stage = 0; fph ^= 1; }
    }
}

// ------------------------------------------------------------ shared-matrix product
// Right-hand sides of one solver share A (complex64).  One launch streams
// every tile of A once: an item is a strip of rows of one group over all
// columns; a stage holds the strip's rows x kGrpCols columns of A (one bulk
// copy per 2 KB row segment) and the x chunks of the group's members that
// take part (2 KB each for the Krylov product, 4 KB of hi/lo pairs for the
// residual).
// Consumer warps own 4 rows x 4 members each and keep, in registers, one
// accumulator per (row, member) across all column chunks; at the strip's
// last chunk they write the members' full-row products (nchunk = 1).
// Krylov product: 16 consumer warps, 32-row strips, 2 stages of 80 KB.
// Refinement residual (twice the registers): 8 warps, 16 rows, 3 x 64 KB.
template <bool EXACT> struct GrpCfg {
    static constexpr int kWarps = EXACT ? 8 : 16;
    static constexpr int kRows = 2 * kWarps;          // 4 rows per warp pair
    static constexpr int kStages = EXACT ? 3 : 2;
    static constexpr int kXBytes = EXACT ? kGrpCols * 16 : kGrpCols * 8;
    static constexpr int kABytes = kRows * kGrpCols * 8;
    static constexpr int kStageBytes = kABytes + kMaxGroup * kXBytes;
    static constexpr int kSmem = kStages * kStageBytes + 512;
};
static_assert(GrpCfg<false>::kSmem <= 227 * 1024 && GrpCfg<true>::kSmem <= 227 * 1024, "shared memory");
static_assert(GrpCfg<false>::kRows == kGrpRowsInner && GrpCfg<true>::kRows == kGrpRowsExact, "plan strip heights");
__host__ __device__ constexpr int grp_smem_bytes(bool exact) {
    return exact ? GrpCfg<true>::kSmem : GrpCfg<false>::kSmem;
}

struct GrpMeta {
    int first, chunk, row0, nrows, len, last, mask, pad;
};

template <bool EXACT>
__global__ void __launch_bounds__(32 * (GrpCfg<EXACT>::kWarps + 1), 1) k_mv_grp(KTable *tb, int kind) {
    extern __shared__ __align__(128) unsigned char smem[];
    using Cfg = GrpCfg<EXACT>;
    constexpr int SB = Cfg::kStageBytes, XB = Cfg::kXBytes, NW = Cfg::kWarps, ROWS = Cfg::kRows;
    constexpr int NS = Cfg::kStages, ASTAGE = Cfg::kABytes;
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + NS * SB);
    GrpMeta *meta = reinterpret_cast<GrpMeta *>(bars + 2 * NS);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + NS);
    if (threadIdx.x == 0) {
        for (int s = 0; s < NS; ++s) {
            mbar_init(full0 + 8 * s, 1);
            mbar_init(empty0 + 8 * s, NW);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __shared__ PlanSmem pl;
    plan_load(tb->gplan[kind], pl);   // includes a block barrier
    int *err = &tb->err;
    // bound of the waits (the drains of in-flight copies keep the full bound)
    const long long lim = (tb->wait_cycles > 0 && ((tb->wait_kinds >> kind) & 1)) ? tb->wait_cycles : kWaitCycles;
    if (warp == NW) {
        // ---------------- producer warp: lane 0 takes the strips and keeps the
        // barriers; lane r < ROWS issues row r's copy, the other copies (the
        // members' x chunks) go round the lanes
        const unsigned kAll = 0xffffffffu;
        const int total = pl.off[pl.n];
        int stage = 0;
        uint32_t eph = 1;
        int issued[NS];
        uint32_t fph[NS];
        for (int q = 0; q < NS; ++q) { issued[q] = 0; fph[q] = 0; }
        bool ok = true;
        while (ok && total > 0) {
            int item = 0;
            if (lane == 0) item = (int)atomicAdd(&tb->mv_ctr[0], 1u);
            item = __shfl_sync(kAll, item, 0);
            if (item >= total) break;
            const int j = plan_find(pl.off, pl.n, item);
            const KGroup g = tb->grp[pl.sys[j]];
            const unsigned mask = tb->gmask[kind][j];
            const KSys &S0 = tb->sys[g.first];
            const int n = S0.n;
            const int row0 = (item - pl.off[j]) * ROWS, nrows = min(ROWS, n - row0);
            const int nck = (n + kGrpCols - 1) / kGrpCols;
            const float2 *A = (const float2 *)S0.A;
            const size_t lda = (size_t)S0.lda;
            const int nmem = __popc(mask & ((1u << g.count) - 1u));
            constexpr int XPER = EXACT ? 2 : 1;   // copies per member and stage
            for (int ck = 0; ck < nck && ok; ++ck) {
                int w = 1;
                if (lane == 0) w = mbar_wait(empty0 + 8 * stage, eph, err, lim);
                if (!__shfl_sync(kAll, w, 0)) { ok = false; break; }
                const int c0 = ck * kGrpCols, len = min(kGrpCols, n - c0), lenp = (len + 1) & ~1;
                const uint32_t xbytes = EXACT ? (uint32_t)XB : (uint32_t)(lenp * 8);
                const uint32_t fb = full0 + 8 * stage;
                if (lane == 0) {
                    GrpMeta mt;
                    mt.first = g.first; mt.chunk = ck; mt.row0 = row0; mt.nrows = nrows; mt.len = len;
                    mt.last = ck == nck - 1; mt.mask = (int)mask; mt.pad = 0;
                    meta[stage] = mt;
                    mbar_expect_tx(fb, (uint32_t)(nrows * lenp * 8) + nmem * xbytes);
                }
                __syncwarp();
                const uint32_t dst = smem_u32(smem + stage * SB);
                if (lane < nrows) bulk_g2s(dst + lane * kGrpCols * 8, A + (size_t)(row0 + lane) * lda + c0, lenp * 8, fb);
                for (int t = lane; t < kMaxGroup * XPER; t += 32) {
                    const int q = t / XPER, h = t - q * XPER;
                    if (q >= g.count || !((mask >> q) & 1)) continue;
                    const uint32_t xd = dst + ASTAGE + q * XB;
                    if (EXACT) {
                        // chunk-permuted (hi, lo) pairs: the stage's even entries, then its odd ones
                        const float4 *base = (const float4 *)tb->sys[g.first + q].xf + (size_t)(c0 & ~(kMvChunk - 1));
                        const int o = (c0 & (kMvChunk - 1)) >> 1;
                        bulk_g2s(xd + h * kGrpCols * 8, base + h * (kMvChunk / 2) + o, kGrpCols * 8, fb);
                    } else {
                        bulk_g2s(xd, (const float2 *)tb->sys[g.first + q].xh + c0, lenp * 8, fb);
                    }
                }
                issued[stage] = 1;
                fph[stage] ^= 1;
                if (++stage == NS) { stage = 0; eph ^= 1; }
            }
        }
        if (lane == 0) {
            if (ok) {
                if (mbar_wait(empty0 + 8 * stage, eph, err, lim)) {
                    meta[stage].first = -1;
                    mbar_arrive(full0 + 8 * stage);
                } else {
                    ok = false;
                }
            }
            if (!ok)
                for (int s = 0; s < NS; ++s)
                    if (issued[s]) mbar_wait(full0 + 8 * s, fph[s] ^ 1, err);
            __threadfence();
            if (atomicAdd(&tb->mv_ctr[1], 1u) == gridDim.x - 1) {
                tb->mv_ctr[0] = 0u;
                tb->mv_ctr[1] = 0u;
                __threadfence();
            }
        }
        return;
    }
    // ---------------- consumers: warp w takes rows 4(w/2) .. 4(w/2)+3 of each
    // strip and members 4(w%2) .. 4(w%2)+3: every A value loaded from shared
    // memory serves 4 members, every x value 4 rows
    constexpr int RW = 4, MW = kMaxGroup / 2;
    float ar[RW][MW], ai[RW][MW], er[RW][MW], ei[RW][MW];
    const int rbase = RW * (warp >> 1), mbase = MW * (warp & 1);
    int stage = 0;
    uint32_t fph = 0;
    while (true) {
        if (!mbar_wait(full0 + 8 * stage, fph, err, lim)) return;
        const GrpMeta mt = meta[stage];
        if (mt.first < 0) return;
        if (mt.chunk == 0) {
#pragma unroll
            for (int r = 0; r < RW; ++r)
#pragma unroll
                for (int q = 0; q < MW; ++q) ar[r][q] = ai[r][q] = er[r][q] = ei[r][q] = 0.f;
        }
        const unsigned char *sb = smem + stage * SB;
        const unsigned mymask = ((unsigned)mt.mask >> mbase) & ((1u << MW) - 1u);
        const int len = mt.len, len2 = len >> 1;
        const float4 *Ab = reinterpret_cast<const float4 *>(sb) + rbase * (kGrpCols / 2);
        if (mymask) {
#pragma unroll 2
            for (int c = lane; c < len2; c += 32) {
                float4 a[RW];
#pragma unroll
                for (int r = 0; r < RW; ++r)
                    a[r] = rbase + r < mt.nrows ? Ab[r * (kGrpCols / 2) + c] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
                for (int q = 0; q < MW; ++q) {
                    if (!((mymask >> q) & 1)) continue;
                    const unsigned char *xq = sb + ASTAGE + (mbase + q) * XB;
                    if (!EXACT) {
                        const float4 xv = reinterpret_cast<const float4 *>(xq)[c];   // hi of entries 2c, 2c + 1
#pragma unroll
                        for (int r = 0; r < RW; ++r) {
                            ar[r][q] = fmaf(a[r].x, xv.x, ar[r][q]); ar[r][q] = fmaf(-a[r].y, xv.y, ar[r][q]);
                            ai[r][q] = fmaf(a[r].x, xv.y, ai[r][q]); ai[r][q] = fmaf(a[r].y, xv.x, ai[r][q]);
                            ar[r][q] = fmaf(a[r].z, xv.z, ar[r][q]); ar[r][q] = fmaf(-a[r].w, xv.w, ar[r][q]);
                            ai[r][q] = fmaf(a[r].z, xv.w, ai[r][q]); ai[r][q] = fmaf(a[r].w, xv.z, ai[r][q]);
                        }
                    } else {
                        const float4 x0 = reinterpret_cast<const float4 *>(xq)[c];
                        const float4 x1 = reinterpret_cast<const float4 *>(xq + kGrpCols * 8)[c];
#pragma unroll
                        for (int r = 0; r < RW; ++r) {
                            acc_exact(ar[r][q], er[r][q], a[r].x, x0.x); acc_exact(ar[r][q], er[r][q], -a[r].y, x0.y);
                            acc_exact(ai[r][q], ei[r][q], a[r].x, x0.y); acc_exact(ai[r][q], ei[r][q], a[r].y, x0.x);
                            er[r][q] = fmaf(a[r].x, x0.z, er[r][q]); er[r][q] = fmaf(-a[r].y, x0.w, er[r][q]);
                            ei[r][q] = fmaf(a[r].x, x0.w, ei[r][q]); ei[r][q] = fmaf(a[r].y, x0.z, ei[r][q]);
                            acc_exact(ar[r][q], er[r][q], a[r].z, x1.x); acc_exact(ar[r][q], er[r][q], -a[r].w, x1.y);
                            acc_exact(ai[r][q], ei[r][q], a[r].z, x1.y); acc_exact(ai[r][q], ei[r][q], a[r].w, x1.x);
                            er[r][q] = fmaf(a[r].z, x1.z, er[r][q]); er[r][q] = fmaf(-a[r].w, x1.w, er[r][q]);
                            ei[r][q] = fmaf(a[r].z, x1.w, ei[r][q]); ei[r][q] = fmaf(a[r].w, x1.z, ei[r][q]);
                        }
                    }
                }
            }
            if ((len & 1) && lane == 0) {   // odd tail: entry len - 1
                float2 b[RW];
#pragma unroll
                for (int r = 0; r < RW; ++r)
                    b[r] = rbase + r < mt.nrows ? reinterpret_cast<const float2 *>(Ab + r * (kGrpCols / 2))[len - 1]
                                                : make_float2(0.f, 0.f);
#pragma unroll
                for (int q = 0; q < MW; ++q) {
                    if (!((mymask >> q) & 1)) continue;
                    const unsigned char *xq = sb + ASTAGE + (mbase + q) * XB;
                    float xr, xi, lr = 0.f, li = 0.f;
                    if (!EXACT) {
                        const float2 xv = reinterpret_cast<const float2 *>(xq)[len - 1];
                        xr = xv.x; xi = xv.y;
                    } else {
                        const float4 x0 = reinterpret_cast<const float4 *>(xq)[(len - 1) >> 1];
                        xr = x0.x; xi = x0.y; lr = x0.z; li = x0.w;
                    }
#pragma unroll
                    for (int r = 0; r < RW; ++r) {
                        if (!EXACT) {
                            ar[r][q] = fmaf(b[r].x, xr, ar[r][q]); ar[r][q] = fmaf(-b[r].y, xi, ar[r][q]);
                            ai[r][q] = fmaf(b[r].x, xi, ai[r][q]); ai[r][q] = fmaf(b[r].y, xr, ai[r][q]);
                        } else {
                            acc_exact(ar[r][q], er[r][q], b[r].x, xr); acc_exact(ar[r][q], er[r][q], -b[r].y, xi);
                            acc_exact(ai[r][q], ei[r][q], b[r].x, xi); acc_exact(ai[r][q], ei[r][q], b[r].y, xr);
                            er[r][q] = fmaf(b[r].x, lr, er[r][q]); er[r][q] = fmaf(-b[r].y, li, er[r][q]);
                            ei[r][q] = fmaf(b[r].x, li, ei[r][q]); ei[r][q] = fmaf(b[r].y, lr, ei[r][q]);
                        }
                    }
                }
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(empty0 + 8 * stage);
        if (mt.last && mymask) {
#pragma unroll
            for (int q = 0; q < MW; ++q) {
                if (!((mymask >> q) & 1)) continue;
                const KSys &S = tb->sys[mt.first + mbase + q];
#pragma unroll
                for (int r = 0; r < RW; ++r) {
                    const double tr = warp_sum_d((double)ar[r][q] + (double)er[r][q]);
                    const double ti = warp_sum_d((double)ai[r][q] + (double)ei[r][q]);
                    if (lane == 0 && rbase + r < mt.nrows) S.mvp[mt.row0 + rbase + r] = make_double2(tr, ti);
                }
            }
        }
        if (++stage == NS) { stage = 0; fph ^= 1; }
    }
}

// ------------------------------------------------------------ shared-matrix product on tensor cores
// The Krylov product of a shared-matrix group as a real GEMM on the tensor
// cores (mma.sync m16n8k8, TF32 inputs, FP32 accumulation, three products
// per step so that the result has FP32 accuracy: A_hi X_hi + A_hi X_lo +
// A_lo X_hi with hi = A rounded to TF32, lo = A - hi).  The complex product
// is real-ified on A's own memory layout: a complex64 row (re, im, re, im,
// ...) is a real row A^ of twice the length, and with
//   X^[2j][r] = re x_j(r), X^[2j+1][r] = -im x_j(r)      (output column r: Re y_r)
//   X^[2j][8+r] = im x_j(r), X^[2j+1][8+r] = re x_j(r)   (output column 8+r: Im y_r)
// Y^ = A^ X^ holds the real and imaginary parts of the 8 members' products.
// The producer is the one of k_mv_grp (32-row strips, stages of 256 columns);
// rows and member x chunks sit at padded strides in shared memory so that the
// fragment loads are free of bank conflicts.  Consumer warp w takes row block
// w & 1 (16 rows) and the slice w >> 1 of each stage's columns.  The MMA
// accumulators hold one stage's partial; each stage's partial is added into
// a float-float (two-sum) accumulator, so the strip's long sum keeps about
// twice-FP32 accuracy; the slice sums of a row block are added in FP64 at
// the end of the strip.
constexpr int kTcRows = kGrpRowsInner;                 // 32
constexpr int kTcRowStride = kGrpCols * 8 + 16;        // bytes, padded row
constexpr int kTcXStride = kGrpCols * 8 + 16;          // bytes, padded member chunk
constexpr int kTcABytes = kTcRows * kTcRowStride;
constexpr int kTcStageBytes = kTcABytes + kMaxGroup * kTcXStride;
constexpr int kTcStages = 2;
constexpr int kTcWarps = 8;                             // consumer warps: 2 row blocks x 4 column slices
constexpr int kTcSlice = kGrpCols / (kTcWarps / 2);      // complex columns of a warp's slice
constexpr int kTcRedBytes = kTcWarps * 16 * 16 * 8;     // per warp a 16 x 16 FP64 tile
constexpr int kTcSmem = kTcStages * kTcStageBytes + kTcRedBytes + 512;
static_assert(kTcSmem <= 227 * 1024, "shared memory");
static_assert(kTcRows == 32 && kTcSlice % 4 == 0 && kTcWarps * 32 >= 256, "row blocks x column slices");

// round to TF32 (nearest, ties away from zero) and the remainder
__device__ __forceinline__ void tf32_split(float v, uint32_t &hi, uint32_t &lo) {
    const uint32_t b = __float_as_uint(v);
    hi = (b + 0x1000u) & 0xffffe000u;
    lo = __float_as_uint(v - __uint_as_float(hi));
}

__device__ __forceinline__ void mma_tf32(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
    asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, "
                 "{%8, %9}, {%0, %1, %2, %3};"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__global__ void __launch_bounds__(32 * (kTcWarps + 1), 1) k_mv_grp_tc(KTable *tb, int kind) {
    if (kind == 0 && tb->grp_umma) return;   // k_mv_grp_umma takes the Krylov products
    extern __shared__ __align__(128) unsigned char smem[];
    double *red = reinterpret_cast<double *>(smem + kTcStages * kTcStageBytes);
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + kTcStages * kTcStageBytes + kTcRedBytes);
    // bars: full[2], empty[2], then the two barriers of the end-of-strip reduction
    GrpMeta *meta = reinterpret_cast<GrpMeta *>(bars + 2 * kTcStages + 2);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + kTcStages);
    const uint32_t redw = smem_u32(bars + 2 * kTcStages), redr = redw + 8;
    if (threadIdx.x == 0) {
        for (int s = 0; s < kTcStages; ++s) {
            mbar_init(full0 + 8 * s, 1);
            mbar_init(empty0 + 8 * s, kTcWarps);
        }
        mbar_init(redw, kTcWarps);
        mbar_init(redr, kTcWarps);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __shared__ PlanSmem pl;
    plan_load(tb->gplan[kind], pl);   // includes a block barrier
    int *err = &tb->err;
    // bound of the waits (the drains of in-flight copies keep the full bound)
    const long long lim = (tb->wait_cycles > 0 && ((tb->wait_kinds >> kind) & 1)) ? tb->wait_cycles : kWaitCycles;
    if (warp == kTcWarps) {
        // ---------------- producer warp: lane 0 takes the strips and keeps the
        // barriers; lane r issues the bulk copy of row r of a stage and lanes
        // 0 .. 7 the members' x chunks (one lane issuing all 40 copies of a
        // stage held the product at about half the HBM bandwidth)
        const unsigned kAll = 0xffffffffu;
        const int total = pl.off[pl.n];
        int stage = 0;
        uint32_t eph = 1;
        int issued[kTcStages] = {0, 0};
        uint32_t fph[kTcStages] = {0, 0};
        bool ok = true;
        while (ok && total > 0) {
            int item = 0;
            if (lane == 0) item = (int)atomicAdd(&tb->mv_ctr[0], 1u);
            item = __shfl_sync(kAll, item, 0);
            if (item >= total) break;
            const int j = plan_find(pl.off, pl.n, item);
            const KGroup g = tb->grp[pl.sys[j]];
            const unsigned mask = tb->gmask[kind][j];
            const KSys &S0 = tb->sys[g.first];
            const int n = S0.n;
            const int row0 = (item - pl.off[j]) * kTcRows, nrows = min(kTcRows, n - row0);
            const int nck = (n + kGrpCols - 1) / kGrpCols;
            const float2 *A = (const float2 *)S0.A;
            const size_t lda = (size_t)S0.lda;
            // this lane's member x array (lanes 0 .. 7), and the member count
            const float2 *xsrc = (lane < g.count && ((mask >> lane) & 1)) ? tb->sys[g.first + lane].xh : nullptr;
            const int nmem = __popc(mask & ((1u << g.count) - 1u));
            for (int ck = 0; ck < nck && ok; ++ck) {
                int w = 1;
                if (lane == 0) w = mbar_wait(empty0 + 8 * stage, eph, err, lim);
                if (!__shfl_sync(kAll, w, 0)) { ok = false; break; }
                const int c0 = ck * kGrpCols, len = min(kGrpCols, n - c0), lenp = (len + 1) & ~1;
                const uint32_t fb = full0 + 8 * stage;
                if (lane == 0) {
                    GrpMeta mt;
                    mt.first = g.first; mt.chunk = ck; mt.row0 = row0; mt.nrows = nrows; mt.len = len;
                    mt.last = ck == nck - 1; mt.mask = (int)mask; mt.pad = 0;
                    meta[stage] = mt;
                    mbar_expect_tx(fb, (uint32_t)((nrows + nmem) * lenp * 8));
                }
                __syncwarp();
                const uint32_t dst = smem_u32(smem + stage * kTcStageBytes);
                if (lane < nrows)
                    bulk_g2s(dst + lane * kTcRowStride, A + (size_t)(row0 + lane) * lda + c0, lenp * 8, fb);
                if (xsrc) bulk_g2s(dst + kTcABytes + lane * kTcXStride, xsrc + c0, lenp * 8, fb);
                issued[stage] = 1;
                fph[stage] ^= 1;
                if (++stage == kTcStages) { stage = 0; eph ^= 1; }
            }
        }
        if (lane == 0) {
            if (ok) {
                if (mbar_wait(empty0 + 8 * stage, eph, err, lim)) {
                    meta[stage].first = -1;
                    mbar_arrive(full0 + 8 * stage);
                } else {
                    ok = false;
                }
            }
            if (!ok)
                for (int s = 0; s < kTcStages; ++s)
                    if (issued[s]) mbar_wait(full0 + 8 * s, fph[s] ^ 1, err);
            __threadfence();
            if (atomicAdd(&tb->mv_ctr[1], 1u) == gridDim.x - 1) {
                tb->mv_ctr[0] = 0u;
                tb->mv_ctr[1] = 0u;
                __threadfence();
            }
        }
        return;
    }
    // ---------------- consumers
    const int gid = lane >> 2, tig = lane & 3;
    const int rb = warp & 1, kq = warp >> 1;   // kq: column slice
    // three independent MMA accumulators per tile (hi*hi, hi*lo, lo*hi), so
    // that consecutive MMAs do not wait on each other
    float dre[3][4], dim[3][4];
    float sh[8], sl[8];   // float-float strip sums of the Re (0-3) and Im (4-7) tiles
    int stage = 0;
    uint32_t fph = 0, rph = 0;
    while (true) {
        if (!mbar_wait(full0 + 8 * stage, fph, err, lim)) return;
        const GrpMeta mt = meta[stage];
        if (mt.first < 0) return;
        if (mt.chunk == 0) {
#pragma unroll
            for (int i = 0; i < 8; ++i) sh[i] = sl[i] = 0.f;
        }
#pragma unroll
        for (int u = 0; u < 3; ++u)
#pragma unroll
            for (int i = 0; i < 4; ++i) dre[u][i] = dim[u][i] = 0.f;
        const unsigned char *sb = smem + stage * kTcStageBytes;
        const float *Ar0 = reinterpret_cast<const float *>(sb + (rb * 16 + gid) * kTcRowStride);
        const float *Ar8 = reinterpret_cast<const float *>(sb + (rb * 16 + gid + 8) * kTcRowStride);
        const bool mem_ok = (mt.mask >> gid) & 1;
        const float2 *xm = reinterpret_cast<const float2 *>(sb + kTcABytes + gid * kTcXStride);
        // this warp's slice of the stage, 4 complex columns per step
#pragma unroll 4
        for (int st4 = 0; st4 < kTcSlice / 4; ++st4) {
            const int j0 = kq * kTcSlice + st4 * 4;
            if (j0 >= mt.len) break;
            // A fragment: real columns 2 j0 + tig and 2 j0 + tig + 4
            const int ka = 2 * j0 + tig, kb = ka + 4;
            const bool va = (ka >> 1) < mt.len, vb = (kb >> 1) < mt.len;
            const float fa0 = va ? Ar0[ka] : 0.f, fa1 = va ? Ar8[ka] : 0.f;
            const float fa2 = vb ? Ar0[kb] : 0.f, fa3 = vb ? Ar8[kb] : 0.f;
            uint32_t ah[4], al[4];
            tf32_split(fa0, ah[0], al[0]);
            tf32_split(fa1, ah[1], al[1]);
            tf32_split(fa2, ah[2], al[2]);
            tf32_split(fa3, ah[3], al[3]);
            // B fragments: member gid, complex entries j0 + (tig >> 1) and j0 + 2 + (tig >> 1)
            const int ja = j0 + (tig >> 1), jb = ja + 2;
            const float2 xa = (mem_ok && ja < mt.len) ? xm[ja] : make_float2(0.f, 0.f);
            const float2 xb = (mem_ok && jb < mt.len) ? xm[jb] : make_float2(0.f, 0.f);
            const bool odd = tig & 1;
            // Re tile: (re, -im) pattern; Im tile: (im, re) pattern
            const float br0 = odd ? -xa.y : xa.x, br1 = odd ? -xb.y : xb.x;
            const float bi0 = odd ? xa.x : xa.y, bi1 = odd ? xb.x : xb.y;
            uint32_t brh0, brl0, brh1, brl1, bih0, bil0, bih1, bil1;
            tf32_split(br0, brh0, brl0);
            tf32_split(br1, brh1, brl1);
            tf32_split(bi0, bih0, bil0);
            tf32_split(bi1, bih1, bil1);
            mma_tf32(dre[0], ah[0], ah[1], ah[2], ah[3], brh0, brh1);
            mma_tf32(dim[0], ah[0], ah[1], ah[2], ah[3], bih0, bih1);
            mma_tf32(dre[1], ah[0], ah[1], ah[2], ah[3], brl0, brl1);
            mma_tf32(dim[1], ah[0], ah[1], ah[2], ah[3], bil0, bil1);
            mma_tf32(dre[2], al[0], al[1], al[2], al[3], brh0, brh1);
            mma_tf32(dim[2], al[0], al[1], al[2], al[3], bih0, bih1);
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(empty0 + 8 * stage);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            float t, e;
            two_sum(sh[i], dre[0][i] + (dre[1][i] + dre[2][i]), t, e);
            sh[i] = t;
            sl[i] += e;
            two_sum(sh[4 + i], dim[0][i] + (dim[1][i] + dim[2][i]), t, e);
            sh[4 + i] = t;
            sl[4 + i] += e;
        }
        if (mt.last) {
            // this warp's 16 x 16 tile (columns 0-7 Re, 8-15 Im) to shared memory;
            // C fragment: rows gid, gid + 8; columns 2 tig, 2 tig + 1
            double *t = red + warp * 256;
            t[gid * 16 + 2 * tig] = (double)sh[0] + (double)sl[0];
            t[gid * 16 + 2 * tig + 1] = (double)sh[1] + (double)sl[1];
            t[(gid + 8) * 16 + 2 * tig] = (double)sh[2] + (double)sl[2];
            t[(gid + 8) * 16 + 2 * tig + 1] = (double)sh[3] + (double)sl[3];
            t[gid * 16 + 8 + 2 * tig] = (double)sh[4] + (double)sl[4];
            t[gid * 16 + 8 + 2 * tig + 1] = (double)sh[5] + (double)sl[5];
            t[(gid + 8) * 16 + 8 + 2 * tig] = (double)sh[6] + (double)sl[6];
            t[(gid + 8) * 16 + 8 + 2 * tig + 1] = (double)sh[7] + (double)sl[7];
            __syncwarp();
            if (lane == 0) mbar_arrive(redw);
            if (!mbar_wait(redw, rph, err, lim)) return;
            // outputs (row block, row, member) = consumer thread index < 256; the
            // sum of the slices of its row block (warps rb, rb + 2, ...)
            const int ot = warp * 32 + lane;
            if (ot < 256) {
                const int orb = ot >> 7, row = (ot >> 3) & 15, q = ot & 7;
                double yr = 0.0, yi = 0.0;
#pragma unroll
                for (int k8 = 0; k8 < kTcWarps / 2; ++k8) {
                    const double *u = red + (orb + 2 * k8) * 256 + row * 16;
                    yr += u[q];
                    yi += u[8 + q];
                }
                const int grow = orb * 16 + row;
                if (grow < mt.nrows && ((mt.mask >> q) & 1)) {
                    double2 *mv = tb->sys[mt.first + q].mvp;
                    if (kind == 0)   // Krylov partials are float (k_dot1)
                        reinterpret_cast<float2 *>(mv)[mt.row0 + grow] = make_float2((float)yr, (float)yi);
                    else
                        mv[mt.row0 + grow] = make_double2(yr, yi);
                }
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(redr);
            if (!mbar_wait(redr, rph, err, lim)) return;   // the tile is free for the next strip
            rph ^= 1;
        }
        if (++stage == kTcStages) { stage = 0; fph ^= 1; }
    }
}


// ------------------------------------------------------------ tcgen05 product
// Krylov product of the shared-matrix groups on the 5th-generation tensor
// cores.  The real-ified product Y^ = A^ X^ (A^: rows of interleaved (re, im)
// complex64 entries, K = 2 n floats; X^: 16 columns, (re, -im) and (im, re)
// patterns of the 8 members' x) is one tcgen05.mma.kind::tf32 chain per
// 128-row strip: M = 128 rows (TMEM lanes), N = 16, K = 8 per instruction,
// FP32 accumulation in TMEM.  TF32 operands carry about 3 digits, the
// accuracy an inner GMRES cycle needs (the refinement residuals keep the
// FP32-accurate products).
// Warp 0: TMA producer.  A comes through the group's tensor map as two
//   32-float x 128-row boxes per stage (128-byte swizzle, the layout the
//   MMA's K-major descriptors read); lanes 0-7 bulk-copy the members' x chunks.
// Warp 1: owns the TMEM allocation; lane 0 issues the MMAs and commits them
//   to the stage's empty barrier (and, at a strip's end, to dfull).
// Warps 2-5: build X^ of each stage in shared memory (K-major, swizzled),
//   and after a strip's last stage read D from TMEM (warp w reads lanes
//   32 (w mod 4) ..) and write the members' row results.
// Every wait is bounded; on expiry the error word is set, copies and MMAs in
// flight are drained, and TMEM is released before the block exits.
constexpr int kUmN = 16;
constexpr int kUmKS = 64;                                  // floats of K per stage
constexpr int kUmStages = 4;
constexpr int kUmASub = kUmRows * 32 * 4;                  // one 128-byte column of A: 16 KB
constexpr int kUmABytes = 2 * kUmASub;
constexpr int kUmBSub = kUmN * 32 * 4;                     // 2 KB
constexpr int kUmBBytes = 2 * kUmBSub;
constexpr int kUmXBytes = kMaxGroup * (kUmKS / 2) * 8;     // 32 complex entries per member
constexpr int kUmStageBytes = kUmABytes + kUmBBytes + kUmXBytes;
constexpr int kUmWarps = 6;
constexpr int kUmSmem = kUmStages * kUmStageBytes + 1024 + 1024;
static_assert(kUmStageBytes % 1024 == 0 && kUmABytes % 1024 == 0, "stage buffers keep the 1024-byte swizzle alignment");
static_assert(kUmSmem <= 227 * 1024, "shared memory");
constexpr uint32_t kUmIdesc = umma::instr_desc(umma::kDF32, umma::kFmtTF32, umma::kFmtTF32, kUmRows, kUmN);

struct UmMeta {
    int first, row0, nrows, k0, len, flags;   // flags: 1 first stage of a strip, 2 last
    unsigned mask;
    int grp;
};

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t mbar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(mbar)
        : "memory");
}
__device__ __forceinline__ void umma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, int acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(d_tmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
        : "memory");
}
__device__ __forceinline__ void umma_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__global__ void __launch_bounds__(32 * kUmWarps, 1) k_mv_grp_umma(KTable *tb) {
    if (!tb->grp_umma) return;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // 1024-byte aligned stage buffers (the swizzle pattern's period)
    const uint32_t raw = smem_u32(smem_raw);
    const uint32_t base = (raw + 1023u) & ~1023u;
    unsigned char *smem = smem_raw + (base - raw);
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + kUmStages * kUmStageBytes);
    // bars: full[4], bready[4], empty[4], dfull, done; then the stage metadata and the TMEM address
    UmMeta *meta = reinterpret_cast<UmMeta *>(bars + 3 * kUmStages + 2);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(meta + kUmStages);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t full0 = smem_u32(bars), bready0 = full0 + 8 * kUmStages, empty0 = bready0 + 8 * kUmStages;
    const uint32_t dfull = empty0 + 8 * kUmStages, done = dfull + 8;
    if (threadIdx.x == 0) {
        for (int s = 0; s < kUmStages; ++s) {
            mbar_init(full0 + 8 * s, 1);
            mbar_init(bready0 + 8 * s, 4);
            mbar_init(empty0 + 8 * s, 1);
        }
        mbar_init(dfull, 1);
        mbar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 32;" ::"r"(smem_u32(tmem_slot))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __shared__ PlanSmem pl;
    plan_load(tb->gplan[0], pl);   // includes a block barrier
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    int *err = &tb->err;
    const long long lim = (tb->wait_cycles > 0 && ((tb->wait_kinds >> 0) & 1)) ? tb->wait_cycles : kWaitCycles;
    const unsigned kAll = 0xffffffffu;

    if (warp == 0) {
        // ---------------- producer
        const int total = pl.off[pl.n];
        int stage = 0;
        uint32_t eph = 1;
        int issued[kUmStages] = {0, 0, 0, 0};
        uint32_t fph[kUmStages] = {0, 0, 0, 0};
        bool ok = true;
        while (ok && total > 0) {
            int item = 0;
            if (lane == 0) item = (int)atomicAdd(&tb->mv_ctr[0], 1u);
            item = __shfl_sync(kAll, item, 0);
            if (item >= total) break;
            const int j = plan_find(pl.off, pl.n, item);
            const int gi = pl.sys[j];
            const KGroup g = tb->grp[gi];
            const unsigned mask = tb->gmask[0][j] & ((1u << g.count) - 1u);
            const int n = tb->sys[g.first].n;
            const int row0 = (item - pl.off[j]) * kUmRows, nrows = min(kUmRows, n - row0);
            const int nks = (2 * n + kUmKS - 1) / kUmKS;
            const float2 *xsrc = (lane < g.count && ((mask >> lane) & 1)) ? tb->sys[g.first + lane].xh : nullptr;
            const int nmem = __popc(mask);
            for (int ks = 0; ks < nks && ok; ++ks) {
                int w = 1;
                if (lane == 0) w = mbar_wait(empty0 + 8 * stage, eph, err, lim);
                if (!__shfl_sync(kAll, w, 0)) { ok = false; break; }
                const int k0 = ks * kUmKS, c0 = k0 >> 1;
                const int len = min(kUmKS / 2, n - c0), lenp = (len + 1) & ~1;
                const uint32_t fb = full0 + 8 * stage;
                const uint32_t sb = base + stage * kUmStageBytes;
                if (lane == 0) {
                    UmMeta mt;
                    mt.first = g.first; mt.row0 = row0; mt.nrows = nrows; mt.k0 = k0; mt.len = len;
                    mt.flags = (ks == 0 ? 1 : 0) | (ks == nks - 1 ? 2 : 0);
                    mt.mask = mask; mt.grp = gi;
                    meta[stage] = mt;
                    // the map was rewritten for this batch through ordinary memory
                    if (ks == 0)
                        asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(
                                         reinterpret_cast<uint64_t>(&tb->gmap[gi]))
                                     : "memory");
                    mbar_expect_tx(fb, (uint32_t)kUmABytes + (uint32_t)(nmem * lenp * 8));
                    // A: two 32-float columns; x is a multiple of 32 floats
                    // (128 bytes), rows and columns past the matrix read zeros
                    tma_load_2d(sb, &tb->gmap[gi], k0, row0, fb);
                    tma_load_2d(sb + kUmASub, &tb->gmap[gi], k0 + 32, row0, fb);
                }
                __syncwarp();
                if (xsrc) bulk_g2s(sb + kUmABytes + kUmBBytes + lane * (kUmKS / 2) * 8, xsrc + c0, lenp * 8, fb);
                issued[stage] = 1;
                fph[stage] ^= 1;
                if (++stage == kUmStages) { stage = 0; eph ^= 1; }
            }
        }
        if (lane == 0) {
            if (ok) {
                if (mbar_wait(empty0 + 8 * stage, eph, err, lim)) {
                    meta[stage].first = -1;
                    mbar_arrive(full0 + 8 * stage);
                } else {
                    ok = false;
                }
            }
            if (!ok)
                for (int s = 0; s < kUmStages; ++s)
                    if (issued[s]) mbar_wait(full0 + 8 * s, fph[s] ^ 1, err);
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer
        if (lane == 0) {
            int stage = 0;
            uint32_t fph = 0;
            while (true) {
                if (!mbar_wait(full0 + 8 * stage, fph, err, lim)) break;
                const UmMeta mt = meta[stage];
                if (mt.first < 0) break;
                if (!mbar_wait(bready0 + 8 * stage, fph, err, lim)) break;
                tc_fence_after();
                const uint32_t sb = base + stage * kUmStageBytes;
#pragma unroll
                for (int sub = 0; sub < 2; ++sub) {
#pragma unroll
                    for (int kk = 0; kk < 4; ++kk) {
                        const uint64_t ad = umma::smem_desc(sb + sub * kUmASub + kk * 32, 16, 1024, umma::kLayout128B);
                        const uint64_t bd =
                            umma::smem_desc(sb + kUmABytes + sub * kUmBSub + kk * 32, 16, 1024, umma::kLayout128B);
                        umma_tf32(tmem, ad, bd, kUmIdesc, ((mt.flags & 1) && sub == 0 && kk == 0) ? 0 : 1);
                    }
                }
                umma_commit(empty0 + 8 * stage);   // the stage's buffers are free once these MMAs finish
                if (mt.flags & 2) umma_commit(dfull);
                if (++stage == kUmStages) { stage = 0; fph ^= 1; }
            }
            // every MMA issued has finished before TMEM is released
            umma_commit(done);
            mbar_wait(done, 0, err);
        }
        __syncwarp();
    } else {
        // ---------------- X^ builders and epilogue (warps 2-5)
        const int t = threadIdx.x - 64;               // 0 .. 127
        const int q4 = warp & 3;                       // TMEM lane quarter of this warp
        const int brow = t >> 3, bq = brow & 7;        // B row: member bq, Re (rows 0-7) or Im (8-15)
        const bool bim = brow >= 8;
        const int kf0 = (t & 7) * 8;                   // this thread's 8 floats of the row
        int stage = 0;
        uint32_t fph = 0, dph = 0;
        while (true) {
            // every lane waits (each acquires the stage), and the warp leaves
            // together if any lane gave up: the epilogue's TMEM load needs
            // the whole warp
            if (!__all_sync(kAll, mbar_wait(full0 + 8 * stage, fph, err, lim))) break;
            const UmMeta mt = meta[stage];
            if (mt.first < 0) break;
            const uint32_t sbo = (uint32_t)stage * kUmStageBytes;
            const float2 *xq = reinterpret_cast<const float2 *>(smem + sbo + kUmABytes + kUmBBytes) + bq * (kUmKS / 2);
            const bool on = (mt.mask >> bq) & 1;
#pragma unroll
            for (int e = 0; e < 8; ++e) {
                const int kf = kf0 + e, jc = kf >> 1, part = kf & 1;
                float v = 0.f;
                if (on && jc < mt.len) {
                    const float2 x = xq[jc];
                    v = bim ? (part ? x.x : x.y) : (part ? -x.y : x.x);
                }
                *reinterpret_cast<float *>(smem + sbo + kUmABytes + (kf >> 5) * kUmBSub +
                                           umma::sw128_offset(brow, kf & 31)) = v;
            }
            // the tensor core reads X^ through the async proxy
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(bready0 + 8 * stage);
            if (mt.flags & 2) {
                // the strip's result: lane l of this warp holds row 32 q4 + l
                if (!__all_sync(kAll, mbar_wait(dfull, dph, err, lim))) break;
                dph ^= 1;
                tc_fence_after();
                uint32_t r[16];
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
                    "%13, %14, %15}, [%16];"
                    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                      "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                      "=r"(r[15])
                    : "r"(umma::tmem_addr(tmem, 32u * q4, 0)));
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                const int row = 32 * q4 + lane;
                if (row < mt.nrows) {
#pragma unroll
                    for (int q = 0; q < kMaxGroup; ++q)
                        if ((mt.mask >> q) & 1)
                            reinterpret_cast<float2 *>(tb->sys[mt.first + q].mvp)[mt.row0 + row] =
                                make_float2(__uint_as_float(r[q]), __uint_as_float(r[8 + q]));
                }
                tc_fence_before();
            }
            if (++stage == kUmStages) { stage = 0; fph ^= 1; }
        }
    }
    __syncthreads();
    tc_fence_after();
    if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 32;" ::"r"(tmem) : "memory");
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&tb->mv_ctr[1], 1u) == gridDim.x - 1) {
            tb->mv_ctr[0] = 0u;
            tb->mv_ctr[1] = 0u;
            __threadfence();
        }
    }
}

// ------------------------------------------------------------ block low-rank product
// Krylov products of systems with a block low-rank copy (KSys::blr_nb > 0,
// compressed by k_blr_aca / k_blr_check; dense blocks in the fp16 copy).
// Persistent grid of 128-thread blocks (8 resident per SM); items (system,
// block row I, chunk c of kMvChunk columns = kBlrPerItem blocks) from the
// queue.  Phase 1: warp w takes the terms w, w + 4, ... of the item's
// compressed blocks, t_l = s_l V_l . x (fp16 factors, x chunk in shared
// memory).  Phase 2a: thread i streams rows i and i + 128 of the dense
// blocks (fp16 row segments, 32-byte loads, one sector each).  Phase 2b:
// thread t takes rows 4 (t & 63) .. + 3 of the compressed blocks with
// 16-byte loads of U_l for every other term; the two term groups are added
// in order through shared memory, then the dense part times the row's scale
// for the chunk.  Sums run in a fixed order; the partial is float, one per
// row and chunk like k_mv_tma's, so k_dot1 sums them unchanged.
constexpr int kBlrRowsPerThread = 2;   // dense rows per thread; more blocks resident per SM
constexpr int kBlrThreads = kBlrB / kBlrRowsPerThread;
constexpr int kBlrTermGroups = kBlrThreads / 64;   // phase 2b: 64 threads x 4 rows per term group
constexpr int kBlrPerItem = kMvChunk / kBlrB;
constexpr int kBlrTermsPerWarp = 4;   // V rows in flight per warp in phase 1
static_assert(kMvChunk % kBlrB == 0, "a chunk holds whole blocks");

// y += a x, a an fp16 pair
__device__ __forceinline__ void cmac_h(float2 &y, unsigned a, float2 x) {
    const float2 av = h2f(a);
    y.x = fmaf(av.x, x.x, y.x);
    y.x = fmaf(-av.y, x.y, y.x);
    y.y = fmaf(av.x, x.y, y.y);
    y.y = fmaf(av.y, x.x, y.y);
}
__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}

__global__ void __launch_bounds__(kBlrThreads, 4 * kBlrRowsPerThread) k_mv_blr(KTable *tb) {
    __shared__ __align__(16) float2 xs[kMvChunk];
    __shared__ __align__(16) float2 ts[kBlrPerItem][kBlrMaxRank];
    __shared__ __align__(16) float2 red[kBlrTermGroups][kBlrB];   // phase 2b: per term group and row
    __shared__ int rk[kBlrPerItem], tsk[kBlrPerItem + 1];
    __shared__ int item_s;
    __shared__ PlanSmem pl;
    plan_load(tb->bplan, pl);   // includes a block barrier
    const int total = pl.off[pl.n];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    while (total > 0) {
        if (threadIdx.x == 0) item_s = (int)atomicAdd(&tb->mv_ctr[0], 1u);
        __syncthreads();
        const int item = item_s;
        if (item >= total) break;
        const int j = plan_find(pl.off, pl.n, item);
        const KSys &S = tb->sys[pl.sys[j]];
        const int local = item - pl.off[j];
        const int n = S.n, nb = S.blr_nb;
        const int I = local / S.nchunk, c = local - I * S.nchunk;
        const int c0 = c * kMvChunk, row0 = I * kBlrB;
        for (int q = threadIdx.x; q < kMvChunk; q += kBlrThreads)
            xs[q] = c0 + q < n ? S.xh[c0 + q] : make_float2(0.f, 0.f);
        if (threadIdx.x == 0) {
            int acc = 0;
            for (int q = 0; q < kBlrPerItem; ++q) {
                const int J = c * kBlrPerItem + q;
                const int r = J < nb ? S.blr_rank[(size_t)I * nb + J] : 0;
                rk[q] = r;
                tsk[q] = acc;
                acc += r > 0 ? r : 0;
            }
            tsk[kBlrPerItem] = acc;
        }
        __syncthreads();
        // phase 1: t_l of the compressed blocks, kBlrTermsPerWarp terms per
        // warp at a time
        const int nt = tsk[kBlrPerItem];
        for (int t0 = warp; t0 < nt; t0 += kBlrTermsPerWarp * (kBlrThreads / 32)) {
            unsigned a[kBlrTermsPerWarp][kBlrB / 32];
            size_t bl[kBlrTermsPerWarp];
            int qq[kBlrTermsPerWarp], ll[kBlrTermsPerWarp];
#pragma unroll
            for (int h = 0; h < kBlrTermsPerWarp; ++h) {
                const int t = min(t0 + h * (kBlrThreads / 32), nt - 1);
                int q = 0;
                while (t >= tsk[q + 1]) ++q;
                qq[h] = q;
                ll[h] = t - tsk[q];
                bl[h] = ((size_t)I * nb + c * kBlrPerItem + q) * kBlrMaxRank + ll[h];
                // lane: entries 2 lane + 64 e' and the next, e' < 4
                const uint2 *v = reinterpret_cast<const uint2 *>(S.blr_V16 + bl[h] * kBlrB);
#pragma unroll
                for (int e = 0; e < kBlrB / 64; ++e) {
                    const uint2 pr = v[lane + 32 * e];
                    a[h][2 * e] = pr.x;
                    a[h][2 * e + 1] = pr.y;
                }
            }
#pragma unroll
            for (int h = 0; h < kBlrTermsPerWarp; ++h) {
                const float4 *xq4 = reinterpret_cast<const float4 *>(xs + qq[h] * kBlrB);
                float sr = 0.f, si = 0.f;
#pragma unroll
                for (int e = 0; e < kBlrB / 64; ++e) {
                    const float4 x2 = xq4[lane + 32 * e];
                    const float2 a0 = h2f(a[h][2 * e]), a1 = h2f(a[h][2 * e + 1]);
                    sr = fmaf(a0.x, x2.x, sr);
                    sr = fmaf(-a0.y, x2.y, sr);
                    si = fmaf(a0.x, x2.y, si);
                    si = fmaf(a0.y, x2.x, si);
                    sr = fmaf(a1.x, x2.z, sr);
                    sr = fmaf(-a1.y, x2.w, sr);
                    si = fmaf(a1.x, x2.w, si);
                    si = fmaf(a1.y, x2.z, si);
                }
                sr = warp_sum_f(sr);
                si = warp_sum_f(si);
                if (lane == 0 && (h == 0 || t0 + h * (kBlrThreads / 32) < nt)) {
                    const float sc = S.blr_scale[bl[h]];
                    ts[qq[h]][ll[h]] = make_float2(sr * sc, si * sc);
                }
            }
        }
        __syncthreads();
        // phase 2a: thread i streams rows i + kBlrThreads r of the dense
        // blocks (fp16 row segments, 32-byte loads)
        float2 yd[kBlrRowsPerThread];
        bool dense = false;
#pragma unroll
        for (int rr = 0; rr < kBlrRowsPerThread; ++rr) yd[rr] = make_float2(0.f, 0.f);
#pragma unroll 1
        for (int q = 0; q < kBlrPerItem; ++q) {
            const int J = c * kBlrPerItem + q;
            if (J >= nb) break;
            if (rk[q] >= 0) continue;
            dense = true;
            const int nc = min(kBlrB, n - J * kBlrB);
            const float2 *xq = xs + q * kBlrB;
#pragma unroll
            for (int rr = 0; rr < kBlrRowsPerThread; ++rr) {
                const int row = row0 + threadIdx.x + rr * kBlrThreads;
                if (row >= n) continue;
                const unsigned *h = reinterpret_cast<const unsigned *>(S.A16) + (size_t)row * S.lda +
                                    (size_t)J * kBlrB;
                if (nc == kBlrB) {
                    const uint4 *h4 = reinterpret_cast<const uint4 *>(h);
#pragma unroll 4
                    for (int g = 0; g < kBlrB / 8; ++g) {
                        const uint4 p0 = h4[2 * g], p1 = h4[2 * g + 1];
                        // x in 16-byte shared loads (two entries each;
                        // every thread reads the same address)
                        const float4 *x4 = reinterpret_cast<const float4 *>(xq + 8 * g);
                        const float4 xa = x4[0], xb = x4[1], xc = x4[2], xd = x4[3];
                        cmac_h(yd[rr], p0.x, make_float2(xa.x, xa.y));
                        cmac_h(yd[rr], p0.y, make_float2(xa.z, xa.w));
                        cmac_h(yd[rr], p0.z, make_float2(xb.x, xb.y));
                        cmac_h(yd[rr], p0.w, make_float2(xb.z, xb.w));
                        cmac_h(yd[rr], p1.x, make_float2(xc.x, xc.y));
                        cmac_h(yd[rr], p1.y, make_float2(xc.z, xc.w));
                        cmac_h(yd[rr], p1.z, make_float2(xd.x, xd.y));
                        cmac_h(yd[rr], p1.w, make_float2(xd.z, xd.w));
                    }
                } else {
                    for (int e = 0; e < nc; ++e) cmac_h(yd[rr], h[e], xq[e]);
                }
            }
        }
        // phase 2b: the compressed blocks; thread t takes rows 4 (t & 63) ..
        // + 3 (16-byte loads of U_l, four rows each) for the terms
        // l = t >> 6 (mod kBlrTermGroups); the term groups meet in shared
        // memory
        {
            constexpr int G = kBlrTermGroups;
            const int rg = threadIdx.x & 63, tg = threadIdx.x >> 6;
            float2 acc[4] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f),
                             make_float2(0.f, 0.f)};
#pragma unroll 1
            for (int q = 0; q < kBlrPerItem; ++q) {
                const int r = rk[q], J = c * kBlrPerItem + q;
                if (J >= nb) break;
                if (r <= 0) continue;
                const uint4 *u = reinterpret_cast<const uint4 *>(S.blr_U16 +
                                                                 ((size_t)I * nb + J) * kBlrMaxRank * kBlrB) + rg;
                int l = tg;
                for (; l + 3 * G < r; l += 4 * G) {
                    uint4 w[4];
#pragma unroll
                    for (int e = 0; e < 4; ++e) w[e] = u[(size_t)(l + G * e) * (kBlrB / 4)];
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const float2 t = ts[q][l + G * e];
                        const float2 p0 = cmulf(h2f(w[e].x), t), p1 = cmulf(h2f(w[e].y), t);
                        const float2 p2 = cmulf(h2f(w[e].z), t), p3 = cmulf(h2f(w[e].w), t);
                        acc[0].x += p0.x; acc[0].y += p0.y;
                        acc[1].x += p1.x; acc[1].y += p1.y;
                        acc[2].x += p2.x; acc[2].y += p2.y;
                        acc[3].x += p3.x; acc[3].y += p3.y;
                    }
                }
                for (; l < r; l += G) {
                    const uint4 w = u[(size_t)l * (kBlrB / 4)];
                    const float2 t = ts[q][l];
                    const float2 p0 = cmulf(h2f(w.x), t), p1 = cmulf(h2f(w.y), t);
                    const float2 p2 = cmulf(h2f(w.z), t), p3 = cmulf(h2f(w.w), t);
                    acc[0].x += p0.x; acc[0].y += p0.y;
                    acc[1].x += p1.x; acc[1].y += p1.y;
                    acc[2].x += p2.x; acc[2].y += p2.y;
                    acc[3].x += p3.x; acc[3].y += p3.y;
                }
            }
            float4 *rd = reinterpret_cast<float4 *>(red[tg] + 4 * rg);
            rd[0] = make_float4(acc[0].x, acc[0].y, acc[1].x, acc[1].y);
            rd[1] = make_float4(acc[2].x, acc[2].y, acc[3].x, acc[3].y);
        }
        __syncthreads();
#pragma unroll
        for (int rr = 0; rr < kBlrRowsPerThread; ++rr) {
            const int il = threadIdx.x + rr * kBlrThreads, row = row0 + il;
            if (row >= n) continue;
            float2 y = red[0][il];
#pragma unroll
            for (int g = 1; g < kBlrTermGroups; ++g) {
                y.x += red[g][il].x;
                y.y += red[g][il].y;
            }
            if (dense) {
                const float sc = S.rs[(size_t)row * S.nchunk + c];
                y.x = fmaf(yd[rr].x, sc, y.x);
                y.y = fmaf(yd[rr].y, sc, y.y);
            }
            reinterpret_cast<float2 *>(S.mvp)[(size_t)c * n + row] = y;
        }
        __syncthreads();   // shared buffers are rewritten by the next item
    }
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&tb->mv_ctr[1], 1u) == gridDim.x - 1) {
            tb->mv_ctr[0] = 0u;
            tb->mv_ctr[1] = 0u;
            __threadfence();
        }
    }
}

// ------------------------------------------------------------ block helpers
// dp[l * nvb + blk] = sum over the block's rows of conj(V_l[row]) w[row], l < nv.
__device__ void block_dots(const double2 *__restrict__ V, long long ldv, int nv, double2 wv, bool ok, int row,
                           double2 *__restrict__ dp, int nvb, int blk, double (*red)[16]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int l0 = 0; l0 < nv; l0 += 8) {
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            double re = 0.0, im = 0.0;
            if (ok && l0 + q < nv) {
                const double2 a = V[(size_t)(l0 + q) * ldv + row];
                re = fma(a.x, wv.x, a.y * wv.y);
                im = fma(a.x, wv.y, -a.y * wv.x);
            }
            re = warp_sum_d(re);
            im = warp_sum_d(im);
            if (lane == 0) {
                red[warp][2 * q] = re;
                red[warp][2 * q + 1] = im;
            }
        }
        __syncthreads();
        if (threadIdx.x < 16) {
            double t = 0.0;
#pragma unroll
            for (int w8 = 0; w8 < 8; ++w8) t += red[w8][threadIdx.x];
            const int q = threadIdx.x >> 1;
            if (l0 + q < nv) reinterpret_cast<double *>(dp + (size_t)(l0 + q) * nvb + blk)[threadIdx.x & 1] = t;
        }
        __syncthreads();
    }
}

// nrmp[blk] = sum over the block's rows of |w|^2
__device__ void block_norm(double2 wv, bool ok, double *__restrict__ nrmp, int blk, double (*red)[16]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double t = ok ? fma(wv.x, wv.x, wv.y * wv.y) : 0.0;
    t = warp_sum_d(t);
    if (lane == 0) red[warp][0] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
#pragma unroll
        for (int w8 = 0; w8 < 8; ++w8) s += red[w8][0];
        nrmp[blk] = s;
    }
    __syncthreads();
}

// sum of the squared-norm partials, in block order
__device__ __forceinline__ double norm_total(const double *__restrict__ nrmp, int nvb) {
    double t = 0.0;
#pragma unroll 8
    for (int c = 0; c < nvb; ++c) t += nrmp[c];
    return t;
}

// The same for the float Krylov basis of complex64 systems: FP32 products
// and sums (GB300's FP64 pipe would bound these loops), one float2 inner-
// product partial per block and vector, the norm partial converted once.
__device__ void block_dots_f(const float2 *__restrict__ V, long long ldv, int nv, float2 wv, bool ok, int row,
                             float2 *__restrict__ dp, int nvb, int blk, float (*red)[16]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int l0 = 0; l0 < nv; l0 += 8) {
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            float re = 0.f, im = 0.f;
            if (ok && l0 + q < nv) {
                const float2 a = V[(size_t)(l0 + q) * ldv + row];
                re = fmaf(a.x, wv.x, a.y * wv.y);
                im = fmaf(a.x, wv.y, -a.y * wv.x);
            }
            re = warp_sum_f(re);
            im = warp_sum_f(im);
            if (lane == 0) {
                red[warp][2 * q] = re;
                red[warp][2 * q + 1] = im;
            }
        }
        __syncthreads();
        if (threadIdx.x < 16) {
            float t = 0.f;
#pragma unroll
            for (int w8 = 0; w8 < 8; ++w8) t += red[w8][threadIdx.x];
            const int q = threadIdx.x >> 1;
            if (l0 + q < nv) reinterpret_cast<float *>(dp + (size_t)(l0 + q) * nvb + blk)[threadIdx.x & 1] = t;
        }
        __syncthreads();
    }
}

__device__ void block_norm_f(float2 wv, bool ok, double *__restrict__ nrmp, int blk, float (*red)[16]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float t = ok ? fmaf(wv.x, wv.x, wv.y * wv.y) : 0.f;
    t = warp_sum_f(t);
    if (lane == 0) red[warp][0] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
        float s = 0.f;
#pragma unroll
        for (int w8 = 0; w8 < 8; ++w8) s += red[w8][0];
        nrmp[blk] = (double)s;
    }
    __syncthreads();
}

// (M^{-1} v)[row] for the thread's own row of a complex128 system: vs holds
// the block's 256 values of v; the thread's 128-row preconditioner block is
// rows (tid & 128) .. +127.  Inverse blocks are stored transposed
// ([col][row]), so the loads coalesce.  (complex64 systems: apply_minv_f.)
__device__ __forceinline__ double2 apply_minv(const void *Minv, int n, int blk, const double2 *vs) {
    const int tid = threadIdx.x;
    const int pb = blk * 2 + (tid >> 7), rr = tid & 127, r0 = pb * kBlock;
    const int nb = min(kBlock, n - r0);
    if (nb <= 0 || rr >= nb) return make_double2(0.0, 0.0);
    const double2 *x = vs + (tid & 128);
    double sr = 0.0, si = 0.0;
    const double2 *M = (const double2 *)Minv + (size_t)pb * kBlock * kBlock;
    for (int c = 0; c < nb; ++c) {
        const double2 m = M[(size_t)c * kBlock + rr];
        const double2 xv = x[c];
        sr = fma(m.x, xv.x, sr); sr = fma(-m.y, xv.y, sr);
        si = fma(m.x, xv.y, si); si = fma(m.y, xv.x, si);
    }
    return make_double2(sr, si);
}

// ------------------------------------------------------------ Arnoldi step
// w = sum of the matvec partials; dpa = V^H w.  complex64 systems keep w and
// V in float (C128 = false).
template <bool C128>
__global__ void __launch_bounds__(kThreads) k_dot1(const KTable *tb) {
    __shared__ double red[8][16];
    __shared__ float redf[8][16];
    for (int it = blockIdx.x; it < tb->vb_total; it += gridDim.x) {
        const int2 bi = tb->vb_items[it];
        const KSys &S = tb->sys[bi.x];
        const KState *st = S.st;
        if (st->phase != kPhaseArnoldi) continue;
        const int n = S.n, blk = bi.y, row = blk * kThreads + threadIdx.x;
        const bool ok = row < n;
        if (!C128) {
            // complex64 products leave float partials: FP32 sum
            float2 wv = make_float2(0.f, 0.f);
            if (ok) {
                const float2 *mp = reinterpret_cast<const float2 *>(S.mvp);
                for (int c = 0; c < S.nchunk; ++c) {
                    const float2 p = mp[(size_t)c * n + row];
                    wv.x += p.x;
                    wv.y += p.y;
                }
                reinterpret_cast<float2 *>(S.w)[row] = wv;
            }
            block_dots_f(reinterpret_cast<const float2 *>(S.V), S.ldv, st->k + 1, wv, ok, row,
                         reinterpret_cast<float2 *>(S.dpa), S.nvb, blk, redf);
        } else {
            double2 wv = make_double2(0.0, 0.0);
            if (ok) {
                for (int c = 0; c < S.nchunk; ++c) {
                    const double2 p = S.mvp[(size_t)c * n + row];
                    wv.x += p.x;
                    wv.y += p.y;
                }
                S.w[row] = wv;
            }
            block_dots(S.V, S.ldv, st->k + 1, wv, ok, row, S.dpa, S.nvb, blk, red);
        }
    }
}

// PASS 1: h = sum(dpa); w -= V h; hsum += h; dpb = V^H w.
// PASS 2: h = sum(dpb); w -= V h; hsum += h; nrmp = |w|^2 partials.
// Systems with one Gram-Schmidt pass (KSys::cgs1) skip PASS 1 and take dpa
// in PASS 2.  complex64 systems (C128 = false): float basis, FP32 sums of
// the block partials and FP32 updates; H accumulates in FP64.
template <int PASS, bool C128>
__global__ void __launch_bounds__(kThreads) k_axpy(const KTable *tb) {
    __shared__ double2 hs[kMaxV];
    __shared__ float2 hsf[kMaxV];
    __shared__ double red[8][16];
    __shared__ float redf[8][16];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int it = blockIdx.x; it < tb->vb_total; it += gridDim.x) {
        const int2 bi = tb->vb_items[it];
        const KSys &S = tb->sys[bi.x];
        const KState *st = S.st;
        if (st->phase != kPhaseArnoldi) continue;
        const int n = S.n, blk = bi.y, row = blk * kThreads + threadIdx.x, nvb = S.nvb;
        const bool ok = row < n;
        const int nv = st->k + 1;
        if (PASS == 1 && S.cgs1) continue;
        const double2 *dp = (PASS == 1 || S.cgs1) ? S.dpa : S.dpb;
        if constexpr (!C128) {
            const float2 *dpf = reinterpret_cast<const float2 *>(dp);
            for (int l = warp; l < nv; l += 8) {
                float re = 0.f, im = 0.f;
                for (int c = lane; c < nvb; c += 32) {
                    const float2 p = dpf[(size_t)l * nvb + c];
                    re += p.x;
                    im += p.y;
                }
                re = warp_sum_f(re);
                im = warp_sum_f(im);
                if (lane == 0) hsf[l] = make_float2(re, im);
            }
            __syncthreads();
            if (blk == 0 && threadIdx.x < nv) {
                double2 hh = S.hsum[threadIdx.x];
                hh.x += (double)hsf[threadIdx.x].x;
                hh.y += (double)hsf[threadIdx.x].y;
                S.hsum[threadIdx.x] = hh;
            }
            float2 wv = make_float2(0.f, 0.f);
            float2 *wf = reinterpret_cast<float2 *>(S.w);
            const float2 *Vf = reinterpret_cast<const float2 *>(S.V);
            if (ok) {
                wv = wf[row];
#pragma unroll 8
                for (int l = 0; l < nv; ++l) {
                    const float2 v = Vf[(size_t)l * S.ldv + row], c = hsf[l];
                    wv.x = fmaf(-c.x, v.x, fmaf(c.y, v.y, wv.x));
                    wv.y = fmaf(-c.x, v.y, fmaf(-c.y, v.x, wv.y));
                }
                wf[row] = wv;
            }
            if (PASS == 1) block_dots_f(Vf, S.ldv, nv, wv, ok, row, reinterpret_cast<float2 *>(S.dpb), nvb, blk, redf);
            else block_norm_f(wv, ok, S.nrmp, blk, redf);
        } else {
            for (int l = warp; l < nv; l += 8) {
                double re = 0.0, im = 0.0;
                for (int c = lane; c < nvb; c += 32) {
                    const double2 p = dp[(size_t)l * nvb + c];
                    re += p.x;
                    im += p.y;
                }
                re = warp_sum_d(re);
                im = warp_sum_d(im);
                if (lane == 0) hs[l] = make_double2(re, im);
            }
            __syncthreads();
            if (blk == 0 && threadIdx.x < nv) {
                double2 hh = S.hsum[threadIdx.x];
                hh.x += hs[threadIdx.x].x;
                hh.y += hs[threadIdx.x].y;
                S.hsum[threadIdx.x] = hh;
            }
            double2 wv = make_double2(0.0, 0.0);
            if (ok) {
                wv = S.w[row];
#pragma unroll 8
                for (int l = 0; l < nv; ++l) {
                    const double2 v = S.V[(size_t)l * S.ldv + row], c = hs[l];
                    wv.x -= c.x * v.x - c.y * v.y;
                    wv.y -= c.x * v.y + c.y * v.x;
                }
                S.w[row] = wv;
            }
            if (PASS == 1) block_dots(S.V, S.ldv, nv, wv, ok, row, S.dpb, nvb, blk, red);
            else block_norm(wv, ok, S.nrmp, blk, red);
        }
    }
}

// RESTART = false: v_{k+1} = w / |w| (phase ARNOLDI).
// RESTART = true:  v_0 = r / beta for systems that have just restarted.
// Then z = M^{-1} v when the system is preconditioned.
// complex64 systems: z = M^{-1} v only feeds the float input of the next
// product, so it is formed in FP32 from a float copy of v (products in FP32,
// chunks of 16 columns added in float-float pairs): no FP64-pipe work per
// column.
__device__ __forceinline__ float2 apply_minv_f(const void *Minv, int n, int blk, const float2 *vf) {
    const int tid = threadIdx.x;
    const int pb = blk * 2 + (tid >> 7), rr = tid & 127, r0 = pb * kBlock;
    const int nb = min(kBlock, n - r0);
    if (nb <= 0 || rr >= nb) return make_float2(0.f, 0.f);
    const float2 *x = vf + (tid & 128);
    const float2 *M = (const float2 *)Minv + (size_t)pb * kBlock * kBlock;
    float sh = 0.f, sl = 0.f, th = 0.f, tl = 0.f;
    if (nb == kBlock) {
        // full block: each chunk's 16 loads issued before its arithmetic
        for (int c0 = 0; c0 < kBlock; c0 += 16) {
            float2 mv[16];
#pragma unroll
            for (int u = 0; u < 16; ++u) mv[u] = M[(size_t)(c0 + u) * kBlock + rr];
            float ar = 0.f, ai = 0.f;
#pragma unroll
            for (int u = 0; u < 16; ++u) {
                const float2 xv = x[c0 + u];
                ar = fmaf(mv[u].x, xv.x, ar); ar = fmaf(-mv[u].y, xv.y, ar);
                ai = fmaf(mv[u].x, xv.y, ai); ai = fmaf(mv[u].y, xv.x, ai);
            }
            float t, e;
            two_sum(sh, ar, t, e); sh = t; sl += e;
            two_sum(th, ai, t, e); th = t; tl += e;
        }
        return make_float2(sh + sl, th + tl);
    }
    for (int c0 = 0; c0 < nb; c0 += 16) {
        float ar = 0.f, ai = 0.f;
        const int ce = min(c0 + 16, nb);
        for (int c = c0; c < ce; ++c) {
            const float2 m = M[(size_t)c * kBlock + rr];
            const float2 xv = x[c];
            ar = fmaf(m.x, xv.x, ar); ar = fmaf(-m.y, xv.y, ar);
            ai = fmaf(m.x, xv.y, ai); ai = fmaf(m.y, xv.x, ai);
        }
        float t, e;
        two_sum(sh, ar, t, e); sh = t; sl += e;
        two_sum(th, ai, t, e); th = t; tl += e;
    }
    return make_float2(sh + sl, th + tl);
}

template <bool C128, bool RESTART>
__global__ void __launch_bounds__(kThreads) k_scale(const KTable *tb) {
    __shared__ double2 vs[kThreads];
    __shared__ float2 vf[kThreads];
    __shared__ double nrm_s;
    for (int it = blockIdx.x; it < tb->vb_total; it += gridDim.x) {
        const int2 bi = tb->vb_items[it];
        const KSys &S = tb->sys[bi.x];
        const KState *st = S.st;
        if (st->phase != kPhaseArnoldi) continue;
        if (RESTART && st->k != 0) continue;
        const int n = S.n, blk = bi.y, row = blk * kThreads + threadIdx.x;
        if (!RESTART) {
            // the norm once per block (same sum, same order as k_givens)
            if (threadIdx.x == 0) nrm_s = norm_total(S.nrmp, S.nvb);
            __syncthreads();
        }
        const double s = RESTART ? 1.0 / st->beta : 1.0 / sqrt(nrm_s);
        const int dst = RESTART ? 0 : st->k + 1;
        // with the window correction, X v goes to pcy and k_pcwin / k_pcfin
        // form the product's input
        if (C128) {
            const double2 *src = RESTART ? S.r : S.w;
            double2 v = make_double2(0.0, 0.0);
            if (row < n) {
                const double2 a = src[row];
                v = make_double2(a.x * s, a.y * s);
                S.V[(size_t)dst * S.ldv + row] = v;
            }
            double2 u = v;   // input of the next product
            if (S.pc) {
                vs[threadIdx.x] = v;
                __syncthreads();
                u = apply_minv(S.Minv, n, blk, vs);
                if (row < n) (S.pcw ? (double2 *)S.pcy : S.z)[row] = u;
            }
        } else {
            // float basis: v = w / |w| in FP32 (v_0 = r / beta from the FP64 r)
            float2 u = make_float2(0.f, 0.f);
            if (row < n) {
                if (RESTART) {
                    const double2 a = S.r[row];
                    u = make_float2((float)(a.x * s), (float)(a.y * s));
                } else {
                    const float2 a = reinterpret_cast<const float2 *>(S.w)[row];
                    const float sf = (float)s;
                    u = make_float2(a.x * sf, a.y * sf);
                }
                reinterpret_cast<float2 *>(S.V)[(size_t)dst * S.ldv + row] = u;
            }
            if (S.pc) {
                vf[threadIdx.x] = u;
                __syncthreads();
                u = apply_minv_f(S.Minv, n, blk, vf);
            }
            if (row < n) (S.pcw ? (float2 *)S.pcy : S.xh)[row] = u;
        }
        __syncthreads();
    }
}

// One thread per system: column k of H from hsum and |w|, the previous
// rotations, the new rotation, |g[k+1]|; ends the cycle (phase UPDATE) when
// the residual estimate reaches the cycle's target, at breakdown, after m
// steps or at the iteration limit.  Clears hsum for the next step.
__device__ void givens_step(const KSys &S) {
    KState *st = S.st;
    const int k = st->k, m = st->m;
    double2 *H = S.H, *cs = S.cs, *sn = S.sn, *g = S.g, *hsum = S.hsum;
    const double hn = sqrt(norm_total(S.nrmp, S.nvb));
    // column k of H from hsum (cleared for the next step) with the previous
    // rotations applied on the way: [a; b] <- [[conj(c), conj(s)], [-s, c]]
    // [a; b]; the running entry stays in registers, the loads do not depend
    // on it
    double2 a = hsum[0];
    hsum[0] = make_double2(0.0, 0.0);
#pragma unroll 4
    for (int l = 0; l < k; ++l) {
        const double2 bb = hsum[l + 1];
        hsum[l + 1] = make_double2(0.0, 0.0);
        const double2 c = cs[l], s = sn[l];
        H[(size_t)l * m + k] = make_double2(c.x * a.x + c.y * a.y + s.x * bb.x + s.y * bb.y,
                                            c.x * a.y - c.y * a.x + s.x * bb.y - s.y * bb.x);
        a = make_double2(-(s.x * a.x - s.y * a.y) + c.x * bb.x - c.y * bb.y,
                         -(s.x * a.y + s.y * a.x) + c.x * bb.y + c.y * bb.x);
    }
    const double den = sqrt(a.x * a.x + a.y * a.y + hn * hn);
    double2 c, s;
    if (den == 0.0) { c = make_double2(1.0, 0.0); s = make_double2(0.0, 0.0); }
    else { c = make_double2(a.x / den, a.y / den); s = make_double2(hn / den, 0.0); }
    cs[k] = c;
    sn[k] = s;
    H[(size_t)k * m + k] = make_double2(c.x * a.x + c.y * a.y + s.x * hn, c.x * a.y - c.y * a.x + s.y * hn);
    const double2 gk = g[k];
    const double2 g1 = make_double2(-(s.x * gk.x - s.y * gk.y), -(s.x * gk.y + s.y * gk.x));
    g[k + 1] = g1;
    g[k] = make_double2(c.x * gk.x + c.y * gk.y, c.x * gk.y - c.y * gk.x);
    const double res = sqrt(g1.x * g1.x + g1.y * g1.y);
    st->k = k + 1;
    st->iters += 1;
    st->n_mv += 1;
    st->res = res;
    if (!(res > st->thr) || hn == 0.0 || !isfinite(res) || k + 1 >= m || st->iters >= st->max_iter)
        st->phase = kPhaseUpdate;
}

// One block of kMaxSys threads, thread t = system t: the Givens step of every
// system in phase ARNOLDI, then, if a system's phase changed, the plans of
// the next Krylov product and of the refinement residual.
__global__ void __launch_bounds__(kMaxSys) k_givens(KTable *tb) {
    __shared__ int changed;   // some system left phase ARNOLDI in this step
    const int b = threadIdx.x;
    if (b == 0) changed = 0;
    __syncthreads();
    if (b < tb->B && tb->sys[b].st->phase == kPhaseArnoldi) {
        givens_step(tb->sys[b]);
        if (tb->sys[b].st->phase != kPhaseArnoldi) atomicOr(&changed, 1);
    }
    __syncthreads();
    // the plans depend only on the systems' phases
    if (changed) {
        plan_build(tb, 0);
        plan_build(tb, 1);
        plan_build(tb, 2);
    }
}

// ------------------------------------------------------------ end of cycle
// y = H^{-1} g (k x k upper triangular), one warp per system.
__global__ void __launch_bounds__(128) k_trisolve(const KTable *tb) {
    __shared__ double2 ys[4][kMaxV];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int b = blockIdx.x * 4 + warp;
    if (b >= tb->B) return;
    const KSys &S = tb->sys[b];
    const KState *st = S.st;
    if (st->phase != kPhaseUpdate || st->k == 0) return;
    const int kk = st->k, m = st->m;
    for (int i = kk - 1; i >= 0; --i) {
        double re = 0.0, im = 0.0;
        for (int l = i + 1 + lane; l < kk; l += 32) {
            const double2 h = S.H[(size_t)i * m + l], yl = ys[warp][l];
            re += h.x * yl.x - h.y * yl.y;
            im += h.x * yl.y + h.y * yl.x;
        }
        re = warp_sum_d(re);
        im = warp_sum_d(im);
        if (lane == 0) {
            const double2 gi = S.g[i], d = S.H[(size_t)i * m + i];
            const double ar = gi.x - re, ai = gi.y - im;
            const double dd = d.x * d.x + d.y * d.y;
            const double2 y = make_double2((ar * d.x + ai * d.y) / dd, (ai * d.x - ar * d.y) / dd);
            ys[warp][i] = y;
            S.y[i] = y;
        }
        __syncwarp();
    }
}

// x += d for the thread's row; complex64 systems also keep the float forms
// of x (first cycle) or d (later cycles) that the residual products read
template <bool C128>
__device__ __forceinline__ void xupdate_finish(const KSys &S, const KState *st, int row, double2 t) {
    double2 xv = S.x[row];
    xv.x += t.x;
    xv.y += t.y;
    S.x[row] = xv;
    if (!C128 && st->cycles == 1) {
        // first residual: (hi, lo) float split of x, stored so that
        // chunk entries 2c and 2c + 1 land in the chunk's first and
        // second half (conflict-free reads in the product)
        const float hr = (float)xv.x, hi = (float)xv.y;
        const int c = row & (kMvChunk - 1);
        S.xf[(size_t)(row - c) + (c & 1) * (kMvChunk / 2) + (c >> 1)] =
            make_float4(hr, hi, (float)(xv.x - (double)hr), (float)(xv.y - (double)hi));
    } else if (!C128) {
        // later residuals: r -= A d, with the float copy of d
        S.xh[row] = make_float2((float)t.x, (float)t.y);
    }
}

// x += M^{-1} (V y)
template <bool C128>
__global__ void __launch_bounds__(kThreads) k_xupdate(const KTable *tb) {
    __shared__ double2 ys[kMaxV];
    __shared__ double2 vs[kThreads];
    __shared__ float2 ysf[kMaxV];
    __shared__ float2 vf[kThreads];
    for (int it = blockIdx.x; it < tb->vb_total; it += gridDim.x) {
        const int2 bi = tb->vb_items[it];
        const KSys &S = tb->sys[bi.x];
        const KState *st = S.st;
        if (st->phase != kPhaseUpdate || st->k == 0) continue;
        const int kk = st->k, n = S.n, blk = bi.y, row = blk * kThreads + threadIdx.x;
        if constexpr (!C128) {
            // float basis: d = M^{-1} V y in FP32, added to x in FP64
            if (threadIdx.x < kk) ysf[threadIdx.x] = make_float2((float)S.y[threadIdx.x].x, (float)S.y[threadIdx.x].y);
            __syncthreads();
            const float2 *Vf = reinterpret_cast<const float2 *>(S.V);
            float2 tf = make_float2(0.f, 0.f);
            if (row < n) {
#pragma unroll 8
                for (int l = 0; l < kk; ++l) {
                    const float2 v = Vf[(size_t)l * S.ldv + row], c = ysf[l];
                    tf.x = fmaf(c.x, v.x, fmaf(-c.y, v.y, tf.x));
                    tf.y = fmaf(c.x, v.y, fmaf(c.y, v.x, tf.y));
                }
            }
            if (S.pc) {
                vf[threadIdx.x] = tf;
                __syncthreads();
                tf = apply_minv_f(S.Minv, n, blk, vf);
            }
            if (row < n) {
                if (!S.pcw) xupdate_finish<false>(S, st, row, make_double2((double)tf.x, (double)tf.y));
                else reinterpret_cast<float2 *>(S.pcy)[row] = tf;   // k_pcfin adds the corrected d
            }
            __syncthreads();
        } else {
            if (threadIdx.x < kk) ys[threadIdx.x] = S.y[threadIdx.x];
            __syncthreads();
            double2 t = make_double2(0.0, 0.0);
            if (row < n) {
#pragma unroll 8
                for (int l = 0; l < kk; ++l) {
                    const double2 v = S.V[(size_t)l * S.ldv + row], c = ys[l];
                    t.x += c.x * v.x - c.y * v.y;
                    t.y += c.x * v.y + c.y * v.x;
                }
            }
            if (S.pc) {
                vs[threadIdx.x] = t;
                __syncthreads();
                t = apply_minv(S.Minv, n, blk, vs);
            }
            if (row < n) {
                if (!S.pcw) xupdate_finish<true>(S, st, row, t);
                else ((double2 *)S.pcy)[row] = t;   // k_pcfin adds the corrected d
            }
            __syncthreads();
        }
    }
}

// ------------------------------------------------------------ window correction
// M v = X (2 I - A_w X) v with X the block-Jacobi inverse and A_w the
// diagonal windows of kPcWin rows of A: after y = X v (k_scale, k_xupdate),
// k_pcwin forms z = A_w y and k_pcfin u = 2 y - X z.  A Neumann step towards
// the inverse of the window blocks: it takes about a sixth of the Krylov
// iterations off block-Jacobi alone on the head-like meshes, for one read
// of the diagonal windows (kPcWin / N of the matrix) per application.
// mode 0: after an Arnoldi step (phase ARNOLDI); 1: after a restart (phase
// ARNOLDI, k = 0); 2: the update at the end of a cycle (phase UPDATE).
__device__ __forceinline__ bool pcw_active(const KSys &S, int mode) {
    const KState *st = S.st;
    if (!S.pcw) return false;
    if (mode == 2) return st->phase == kPhaseUpdate && st->k != 0;
    return st->phase == kPhaseArnoldi && (mode == 0 || st->k == 0);
}

constexpr int kPcRows = 32;                  // rows per k_pcwin item
constexpr int kPcItems = kThreads / kPcRows; // items per vector block
static_assert(kPcWin % kThreads == 0, "windows hold whole vector blocks");
static_assert(kPcWin == kMvChunk, "a window is one column chunk: one fp16 segment scale per row");

__device__ __forceinline__ void cmac(float &sr, float &si, float2 a, float2 y) {
    sr = fmaf(a.x, y.x, sr); sr = fmaf(-a.y, y.y, sr);
    si = fmaf(a.x, y.y, si); si = fmaf(a.y, y.x, si);
}

// z = A_w y, one warp per row; the window's y staged in shared memory.
// Reads the fp16 copy of A when the system keeps one (scaled by the row's
// power of two), else the complex64 or complex128 matrix.
template <bool C128>
__global__ void __launch_bounds__(kThreads) k_pcwin(const KTable *tb, int mode) {
    __shared__ __align__(16) double2 ysh[kPcWin];
    if (!tb->pcw_any) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int it = blockIdx.x; it < tb->vb_total * kPcItems; it += gridDim.x) {
        const int2 bi = tb->vb_items[it / kPcItems];
        const KSys &S = tb->sys[bi.x];
        if (!pcw_active(S, mode)) continue;
        const int n = S.n, r0 = bi.y * kThreads + (it % kPcItems) * kPcRows;
        if (r0 >= n) continue;
        const int c0 = r0 / kPcWin * kPcWin, nw = min(kPcWin, n - c0);
        const int r1 = min(r0 + kPcRows, n);
        __syncthreads();   // the previous item's rows are done with ysh
        if (C128) {
            const double2 *y = (const double2 *)S.pcy + c0;
            for (int c = threadIdx.x; c < nw; c += kThreads) ysh[c] = y[c];
        } else {
            const float2 *y = (const float2 *)S.pcy + c0;
            float2 *yf = reinterpret_cast<float2 *>(ysh);
            for (int c = threadIdx.x; c < nw; c += kThreads) yf[c] = y[c];
        }
        __syncthreads();
        for (int r = r0 + warp; r < r1; r += kThreads / 32) {
            if (C128) {
                const double2 *a = (const double2 *)S.A + (size_t)r * S.lda + c0;
                double sr = 0.0, si = 0.0;
#pragma unroll 4
                for (int c = lane; c < nw; c += 32) {
                    const double2 av = a[c], yv = ysh[c];
                    sr = fma(av.x, yv.x, sr); sr = fma(-av.y, yv.y, sr);
                    si = fma(av.x, yv.y, si); si = fma(av.y, yv.x, si);
                }
                sr = warp_sum_d(sr);
                si = warp_sum_d(si);
                if (lane == 0) ((double2 *)S.pcz)[r] = make_double2(sr, si);
            } else {
                const float2 *yf = reinterpret_cast<const float2 *>(ysh);
                float sr = 0.f, si = 0.f, scale = 1.f;
                if (S.A16) {
                    // 16-byte loads of 4 entries; full windows unrolled
                    const __half2 *a = (const __half2 *)S.A16 + (size_t)r * S.lda + c0;
                    if (nw == kPcWin) {
                        uint4 q[kPcWin / 128];
#pragma unroll
                        for (int p = 0; p < kPcWin / 128; ++p) q[p] = reinterpret_cast<const uint4 *>(a)[lane + 32 * p];
#pragma unroll
                        for (int p = 0; p < kPcWin / 128; ++p) {
                            const int c = 4 * (lane + 32 * p);
                            const __half2 *h = reinterpret_cast<const __half2 *>(&q[p]);
#pragma unroll
                            for (int e = 0; e < 4; ++e) cmac(sr, si, __half22float2(h[e]), yf[c + e]);
                        }
                    } else {
                        for (int c = lane; c < nw; c += 32) cmac(sr, si, __half22float2(a[c]), yf[c]);
                    }
                    scale = S.rs[(size_t)r * mv_chunks(n) + c0 / kMvChunk];
                } else {
                    const float2 *a = (const float2 *)S.A + (size_t)r * S.lda + c0;
                    if (nw == kPcWin) {
                        float4 q[kPcWin / 64];
#pragma unroll
                        for (int p = 0; p < kPcWin / 64; ++p) q[p] = reinterpret_cast<const float4 *>(a)[lane + 32 * p];
#pragma unroll
                        for (int p = 0; p < kPcWin / 64; ++p) {
                            const int c = 2 * (lane + 32 * p);
                            cmac(sr, si, make_float2(q[p].x, q[p].y), yf[c]);
                            cmac(sr, si, make_float2(q[p].z, q[p].w), yf[c + 1]);
                        }
                    } else {
                        for (int c = lane; c < nw; c += 32) cmac(sr, si, a[c], yf[c]);
                    }
                }
                sr = warp_sum_f(sr);
                si = warp_sum_f(si);
                if (lane == 0) ((float2 *)S.pcz)[r] = make_float2(sr * scale, si * scale);
            }
        }
    }
}

// u = 2 y - X z: the product's input (mode 0, 1) or the cycle's update of x
// (mode 2).
template <bool C128>
__global__ void __launch_bounds__(kThreads) k_pcfin(const KTable *tb, int mode) {
    __shared__ double2 vs[kThreads];
    __shared__ float2 vf[kThreads];
    if (!tb->pcw_any) return;
    for (int it = blockIdx.x; it < tb->vb_total; it += gridDim.x) {
        const int2 bi = tb->vb_items[it];
        const KSys &S = tb->sys[bi.x];
        if (!pcw_active(S, mode)) continue;
        const int n = S.n, blk = bi.y, row = blk * kThreads + threadIdx.x;
        const bool ok = row < n;
        if (C128) {
            const double2 *Y = (const double2 *)S.pcy, *Z = (const double2 *)S.pcz;
            vs[threadIdx.x] = ok ? Z[row] : make_double2(0.0, 0.0);
            __syncthreads();
            const double2 q = apply_minv(S.Minv, n, blk, vs);
            if (ok) {
                const double2 y = Y[row];
                const double2 u = make_double2(2.0 * y.x - q.x, 2.0 * y.y - q.y);
                if (mode == 2) xupdate_finish<true>(S, S.st, row, u);
                else S.z[row] = u;
            }
        } else {
            const float2 *Y = (const float2 *)S.pcy, *Z = (const float2 *)S.pcz;
            vf[threadIdx.x] = ok ? Z[row] : make_float2(0.f, 0.f);
            __syncthreads();
            const float2 q = apply_minv_f(S.Minv, n, blk, vf);
            if (ok) {
                const float2 y = Y[row];
                const float2 u = make_float2(2.f * y.x - q.x, 2.f * y.y - q.y);
                if (mode == 2) xupdate_finish<false>(S, S.st, row, make_double2((double)u.x, (double)u.y));
                else S.xh[row] = u;
            }
        }
        __syncthreads();
    }
}

// r = b - A x, or r - A d (complex64 after the first cycle), or r = b before
// the first cycle; |r|^2 partials
__global__ void __launch_bounds__(kThreads) k_resid(const KTable *tb) {
    __shared__ double red[8][16];
    for (int it = blockIdx.x; it < tb->vb_total; it += gridDim.x) {
        const int2 bi = tb->vb_items[it];
        const KSys &S = tb->sys[bi.x];
        const KState *st = S.st;
        if (st->phase != kPhaseUpdate) continue;
        const int n = S.n, blk = bi.y, row = blk * kThreads + threadIdx.x;
        const bool ok = row < n;
        double2 r = make_double2(0.0, 0.0);
        if (ok) {
            // complex64 after the first cycle: recursive update r -= A d
            r = (tb->prec == 1 && st->cycles >= 2) ? S.r[row] : S.b[row];
            if (st->cycles > 0) {
                double ax = 0.0, ay = 0.0;
                for (int c = 0; c < S.nchunk; ++c) {
                    const double2 p = S.mvp[(size_t)c * n + row];
                    ax += p.x;
                    ay += p.y;
                }
                r.x -= ax;
                r.y -= ay;
            }
            S.r[row] = r;
        }
        block_norm(r, ok, S.nrmp, blk, red);
    }
}

// One thread per system: convergence decision after a cycle (or the initial
// residual), then the restart: g = beta e_1, hsum = 0, the cycle's target.
__device__ void decide_step(const KSys &S) {
    KState *st = S.st;
    const double beta = sqrt(norm_total(S.nrmp, S.nvb));
    if (st->cycles == 0) {
        st->bnorm = beta;
        st->beta = beta;
        if (beta == 0.0) {   // zero right-hand side: x = 0
            st->rel = 0.0;
            st->result = kResConverged;
            st->phase = kPhaseFinished;
            return;
        }
        st->rel = 1.0;
        if (!isfinite(beta)) {
            st->result = kResBreakdown;
            st->phase = kPhaseFinished;
            return;
        }
    } else {
        st->n_mv += 1;   // the refinement residual
        st->prev_beta = st->beta;
        st->beta = beta;
        const double rel = beta / st->bnorm;
        st->rel = rel;
        int res = kResRunning;
        if (!isfinite(rel)) res = kResBreakdown;
        else if (rel <= st->tol) res = kResConverged;
        else if (st->iters >= st->max_iter) res = kResMaxIter;
        else if (st->floor_rel > 0.0 && st->cycles > 2 && beta > 0.9 * st->prev_beta) res = kResStagnated;
        if (res != kResRunning) {
            st->result = res;
            st->phase = kPhaseFinished;
            return;
        }
    }
    const int m = st->m;
    st->cycles += 1;
    st->k = 0;
    st->thr = fmax(st->tol * st->bnorm, st->floor_rel * beta);
    S.g[0] = make_double2(beta, 0.0);
    for (int l = 1; l <= m; ++l) S.g[l] = make_double2(0.0, 0.0);
    for (int l = 0; l <= m; ++l) S.hsum[l] = make_double2(0.0, 0.0);
    st->phase = kPhaseArnoldi;
}

// One block of kMaxSys threads: convergence decision after a cycle (or the
// initial residual) and the restart of every system in phase UPDATE, then the
// plans from the new phases (k_givens rebuilds them only when a phase changes
// in its step).
__global__ void __launch_bounds__(kMaxSys) k_decide(KTable *tb) {
    const int b = threadIdx.x;
    if (b < tb->B && tb->sys[b].st->phase == kPhaseUpdate) decide_step(tb->sys[b]);
    __syncthreads();
    plan_build(tb, 0);
    plan_build(tb, 1);
    plan_build(tb, 2);
}

// Both plans from the current phases (after the host rewrote the table).
__global__ void __launch_bounds__(kMaxSys) k_plans(KTable *tb) {
    plan_build(tb, 0);
    plan_build(tb, 1);
    plan_build(tb, 2);
}

int g_mv_grid[2] = {0, 0};
int g_vec_grid = 0;
int g_pcw_grid = 0;   // k_pcwin: every block it can keep resident (loads in flight)
int g_blr_grid = 0;   // k_mv_blr: every block it can keep resident
std::atomic<long long> g_launches{0};

}  // namespace

void count_launches(long long k) { g_launches.fetch_add(k, std::memory_order_relaxed); }
long long launches() { return g_launches.load(std::memory_order_relaxed); }

cudaError_t krylov_prepare() {
    static std::once_flag once;
    static cudaError_t err = cudaSuccess;
    std::call_once(once, [] {
        int dev = 0, sms = 0, per = 0;
        err = cudaGetDevice(&dev);
        if (err == cudaSuccess) err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
        if (err == cudaSuccess)
            err = cudaFuncSetAttribute(k_mv_tma<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       tma_smem_bytes(false));
        if (err == cudaSuccess)
            err = cudaFuncSetAttribute(k_mv_tma<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       tma_smem_bytes(true));
        if (err == cudaSuccess)
            err = cudaFuncSetAttribute(k_mv_grp<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       grp_smem_bytes(false));
        if (err == cudaSuccess)
            err = cudaFuncSetAttribute(k_mv_grp<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       grp_smem_bytes(true));
        if (err == cudaSuccess)
            err = cudaFuncSetAttribute(k_mv_grp_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem);
        if (err == cudaSuccess)
            err = cudaFuncSetAttribute(k_mv_grp_umma, cudaFuncAttributeMaxDynamicSharedMemorySize, kUmSmem);
        g_mv_grid[1] = sms;   // one bulk-copy block per SM
        if (err == cudaSuccess) err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_mv64<false>, 256, 0);
        g_mv_grid[0] = sms * (per > 0 ? per : 1);
        // vector kernels: as many blocks as stay resident, so that a batch's
        // row blocks are all in flight at once (their loops are latency bound)
        per = 0;
        if (err == cudaSuccess)
            err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_scale<false, false>, kThreads, 0);
        g_vec_grid = sms * (per > 2 ? per : 2);
        per = 0;
        if (err == cudaSuccess) err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_pcwin<false>, kThreads, 0);
        g_pcw_grid = sms * (per > 0 ? per : 1);
        per = 0;
        if (err == cudaSuccess) err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_mv_blr, kBlrThreads, 0);
        g_blr_grid = sms * (per > 0 ? per : 1);
    });
    return err;
}

bool group_product_umma() {
    const char *v = std::getenv("BEM_GB300_GROUP_PRODUCT");
    return !(v && std::strcmp(v, "mma") == 0);
}

cudaError_t launch_product(KTable *d_tab, int prec, cudaStream_t st) {
    if (!g_vec_grid) return cudaErrorNotReady;   // krylov_prepare() first
    constexpr int kTmaThreads = 32 * (kTmaConsumers + 1);
    if (prec == 0) k_mv64<false><<<g_mv_grid[0], 256, 0, st>>>(d_tab, 0);
    else k_mv_tma<false><<<g_mv_grid[1], kTmaThreads, tma_smem_bytes(false), st>>>(d_tab, 0);
    return cudaGetLastError();
}

cudaError_t launch_plans(KTable *d_tab, cudaStream_t st) {
    count_launches(1);
    k_plans<<<1, kMaxSys, 0, st>>>(d_tab);
    return cudaGetLastError();
}

// the two launches of the preconditioner's window correction
static void pc_window(bool c128, const KTable *d_tab, int mode, int gv, cudaStream_t st) {
    if (c128) {
        k_pcwin<true><<<g_pcw_grid, kThreads, 0, st>>>(d_tab, mode);
        k_pcfin<true><<<gv, kThreads, 0, st>>>(d_tab, mode);
    } else {
        k_pcwin<false><<<g_pcw_grid, kThreads, 0, st>>>(d_tab, mode);
        k_pcfin<false><<<gv, kThreads, 0, st>>>(d_tab, mode);
    }
}

cudaError_t launch_krylov_body(int prec, const KTable *d_tab, cudaEvent_t *mv_ev, cudaStream_t st,
                               int *launches_out, bool groups, bool blr, bool dense) {
    KTable *tb = const_cast<KTable *>(d_tab);
    const bool c128 = prec == 0;
    if (!g_vec_grid) return cudaErrorNotReady;   // krylov_prepare() first
    const int gmv = g_mv_grid[c128 ? 0 : 1], gv = g_vec_grid;
    int nl = 0;
    cudaError_t e = cudaSuccess;
    constexpr int kTmaThreads = 32 * (kTmaConsumers + 1);
    for (int q = 0; q < kSteps; ++q) {
        if (mv_ev) cudaEventRecordWithFlags(mv_ev[2 * q], st, cudaEventRecordExternal);
        if (c128) k_mv64<false><<<gmv, 256, 0, st>>>(tb, 0);
        else {
            if (dense) k_mv_tma<false><<<gmv, kTmaThreads, tma_smem_bytes(false), st>>>(tb, 0);
            else --nl;   // counted with the step's 8 below
            if (groups) {
                k_mv_grp_tc<<<gmv, 32 * (kTcWarps + 1), kTcSmem, st>>>(tb, 0);
                k_mv_grp_umma<<<gmv, 32 * kUmWarps, kUmSmem, st>>>(tb);
                nl += 2;
            }
            if (blr) {
                k_mv_blr<<<g_blr_grid, kBlrThreads, 0, st>>>(tb);
                ++nl;
            }
        }
        if (mv_ev) cudaEventRecordWithFlags(mv_ev[2 * q + 1], st, cudaEventRecordExternal);
        if (c128) {
            k_dot1<true><<<gv, kThreads, 0, st>>>(d_tab);
            k_axpy<1, true><<<gv, kThreads, 0, st>>>(d_tab);
            k_axpy<2, true><<<gv, kThreads, 0, st>>>(d_tab);
        } else {
            k_dot1<false><<<gv, kThreads, 0, st>>>(d_tab);
            k_axpy<1, false><<<gv, kThreads, 0, st>>>(d_tab);
            k_axpy<2, false><<<gv, kThreads, 0, st>>>(d_tab);
        }
        if (c128) k_scale<true, false><<<gv, kThreads, 0, st>>>(d_tab);
        else k_scale<false, false><<<gv, kThreads, 0, st>>>(d_tab);
        pc_window(c128, d_tab, 0, gv, st);
        k_givens<<<1, kMaxSys, 0, st>>>(tb);
        nl += 8;
    }
    k_trisolve<<<(kMaxSys + 3) / 4, 128, 0, st>>>(d_tab);
    if (c128) k_xupdate<true><<<gv, kThreads, 0, st>>>(d_tab);
    else k_xupdate<false><<<gv, kThreads, 0, st>>>(d_tab);
    pc_window(c128, d_tab, 2, gv, st);
    if (mv_ev) cudaEventRecordWithFlags(mv_ev[2 * kSteps], st, cudaEventRecordExternal);
    if (c128) k_mv64<true><<<gmv, 256, 0, st>>>(tb, 1);
    else {
        // first-cycle residuals with error-free products, then the recursive updates
        k_mv_tma<true><<<gmv, kTmaThreads, tma_smem_bytes(true), st>>>(tb, 1);
        if (groups) k_mv_grp<true><<<gmv, 32 * (GrpCfg<true>::kWarps + 1), grp_smem_bytes(true), st>>>(tb, 1);
        k_mv_tma<false><<<gmv, kTmaThreads, tma_smem_bytes(false), st>>>(tb, 2);
        if (groups) k_mv_grp_tc<<<gmv, 32 * (kTcWarps + 1), kTcSmem, st>>>(tb, 2);
        nl += groups ? 3 : 1;
    }
    if (mv_ev) cudaEventRecordWithFlags(mv_ev[2 * kSteps + 1], st, cudaEventRecordExternal);
    k_resid<<<gv, kThreads, 0, st>>>(d_tab);
    k_decide<<<1, kMaxSys, 0, st>>>(tb);
    if (c128) k_scale<true, true><<<gv, kThreads, 0, st>>>(d_tab);
    else k_scale<false, true><<<gv, kThreads, 0, st>>>(d_tab);
    pc_window(c128, d_tab, 1, gv, st);
    nl += 10;
    e = cudaGetLastError();
    if (launches_out) *launches_out = nl;
    return e;
}

}  // namespace bem
