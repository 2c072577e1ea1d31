// bem_api.cu - the C ABI of include/bem_gb300.h: handles, device memory,
// HBM admission and the per-frequency sequence (assembly, solve, projection)
// for one solver or a batch of solvers.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <unordered_map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/bem_gb300.h"
#include "bem_engine.h"
#include "bem_internal.h"
#include "bem_solver.h"

using cd = std::complex<double>;

thread_local std::string g_err;

namespace bem {

bem_status fail(bem_status st, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    return st;
}

}  // namespace bem

using bem::fail;
using bem::round_up;

namespace {

#define CU(call)                                                                                 \
    do {                                                                                         \
        cudaError_t e_ = (call);                                                                 \
        if (e_ != cudaSuccess)                                                                   \
            return fail(BEM_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
    } while (0)

std::mutex g_init_mu;
bool g_init_done[64];

bem_status ensure_device_init() {
    int dev = 0;
    CU(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_init_mu);
    if (dev < 0 || dev >= 64) return fail(BEM_ERR_INVALID, "device index %d out of range", dev);
    if (!g_init_done[dev]) {
        CU(bem::init_device_tables());
        g_init_done[dev] = true;
    }
    return BEM_OK;
}

template <typename T> cudaError_t dalloc(T **p, size_t count) {
    *p = nullptr;
    if (count == 0) return cudaSuccess;
    return bem::dev_malloc((void **)p, count * sizeof(T));
}


}  // namespace


namespace {

// Centre, unit normal at the centre and area with NumCalc's formulas
// (NC_Input.cpp:522-602 with NC_3dFunctions.cpp:95-178).  This translation
// unit's host code is compiled with -ffp-contract=off so that the products
// and sums round as in the reference's x86 build.
void element_geometry(int nv, const double p[4][3], double c[3], double nrm[3], double *area) {
    double s, t, are0, sh[4], ds[4], dt[4];
    if (nv == 3) {
        s = t = 1.0 / 3.0; are0 = 0.5;
        sh[0] = s; sh[1] = t; sh[2] = 1.0 - s - t;
        ds[0] = 1.0; ds[1] = 0.0; ds[2] = -1.0;
        dt[0] = 0.0; dt[1] = 1.0; dt[2] = -1.0;
    } else {
        s = t = 0.0; are0 = 4.0;
        double s1 = 0.25 * (s + 1.0), s2 = 0.25 * (s - 1.0), t1 = t + 1.0, t2 = t - 1.0;
        sh[0] = s1 * t1; sh[1] = -s2 * t1; sh[2] = s2 * t2; sh[3] = -s1 * t2;
        ds[0] = 0.25 * (t + 1.0); ds[2] = 0.25 * (t - 1.0); ds[1] = -ds[0]; ds[3] = -ds[2];
        dt[0] = 0.25 * (s + 1.0); dt[2] = 0.25 * (s - 1.0); dt[1] = -dt[2]; dt[3] = -dt[0];
    }
    double dxs[3], dxt[3];
    for (int k = 0; k < 3; ++k) {
        c[k] = 0.0; dxs[k] = 0.0; dxt[k] = 0.0;
        for (int a = 0; a < nv; ++a) {
            c[k] += sh[a] * p[a][k];
            dxs[k] += ds[a] * p[a][k];
            dxt[k] += dt[a] * p[a][k];
        }
    }
    double n0 = dxs[1] * dxt[2] - dxt[1] * dxs[2];
    double n1 = dxs[2] * dxt[0] - dxt[2] * dxs[0];
    double n2 = dxs[0] * dxt[1] - dxt[0] * dxs[1];
    double len = std::sqrt(n0 * n0 + n1 * n1 + n2 * n2);
    nrm[0] = n0 / len; nrm[1] = n1 / len; nrm[2] = n2 / len;
    *area = len * are0;
}

// Morton (Z-order) key of a point quantised to 21 bits per axis.
uint64_t spread3(uint64_t v) {
    v &= 0x1fffff;
    v = (v | v << 32) & 0x1f00000000ffffULL;
    v = (v | v << 16) & 0x1f0000ff0000ffULL;
    v = (v | v << 8) & 0x100f00f00f00f00fULL;
    v = (v | v << 4) & 0x10c30c30c30c30c3ULL;
    v = (v | v << 2) & 0x1249249249249249ULL;
    return v;
}

}  // namespace

namespace bem {

// Byte layout of the block (256-byte aligned pieces): the matrix and what
// the right-hand sides share, then the per-right-hand-side buffers (Krylov
// workspace, projection scratch, boundary values and sources) of n_rhs
// right-hand sides.  base == nullptr only sizes it.  extra (n_rhs - 1
// entries) receives right-hand sides 1..n_rhs-1, whose shared fields repeat
// those of *o.
// ---------------------------------------------------------------- device memory cache
namespace {
struct DevCache {
    std::mutex mu;
    bool enabled = true;
    std::unordered_map<void *, std::pair<int, size_t>> live;   // block -> (device, bytes)
    std::map<int, std::multimap<size_t, void *>> idle;          // per device: bytes -> block
    std::map<int, size_t> idle_bytes;
};
DevCache &dev_cache() {
    static DevCache *c = [] {
        DevCache *d = new DevCache();   // never destroyed: blocks may outlive static destructors
        const char *v = std::getenv("BEM_GB300_CACHE");
        d->enabled = !(v && std::string(v) == "0");
        return d;
    }();
    return *c;
}
}  // namespace

cudaError_t dev_malloc(void **p, size_t bytes) {
    *p = nullptr;
    if (bytes == 0) return cudaSuccess;
    const size_t gran = (size_t)2 << 20;
    const size_t want = (bytes + gran - 1) / gran * gran;
    int dev = 0;
    cudaGetDevice(&dev);
    DevCache &C = dev_cache();
    if (C.enabled) {
        std::lock_guard<std::mutex> g(C.mu);
        auto &m = C.idle[dev];
        auto it = m.lower_bound(want);
        if (it != m.end() && it->first <= want + want / 8) {
            *p = it->second;
            C.live[*p] = {dev, it->first};
            C.idle_bytes[dev] -= it->first;
            m.erase(it);
            return cudaSuccess;
        }
    }
    cudaError_t e = cudaMalloc(p, want);
    if (e == cudaErrorMemoryAllocation && C.enabled) {
        cudaGetLastError();
        dev_release_cached(dev);
        e = cudaMalloc(p, want);
    }
    if (e == cudaSuccess) {
        std::lock_guard<std::mutex> g(C.mu);
        C.live[*p] = {dev, want};
    }
    return e;
}

void dev_free(void *p) {
    if (!p) return;
    DevCache &C = dev_cache();
    std::unique_lock<std::mutex> g(C.mu);
    auto it = C.live.find(p);
    if (it == C.live.end() || !C.enabled) {
        if (it != C.live.end()) C.live.erase(it);
        g.unlock();
        cudaFree(p);
        return;
    }
    const int dev = it->second.first;
    const size_t bytes = it->second.second;
    C.live.erase(it);
    g.unlock();
    // as cudaFree: no work still in flight may touch the block when it is reused
    int cur = 0;
    cudaGetDevice(&cur);
    if (cur != dev) cudaSetDevice(dev);
    cudaDeviceSynchronize();
    if (cur != dev) cudaSetDevice(cur);
    g.lock();
    C.idle[dev].emplace(bytes, p);
    C.idle_bytes[dev] += bytes;
}

size_t dev_cached_bytes(int device) {
    DevCache &C = dev_cache();
    std::lock_guard<std::mutex> g(C.mu);
    auto it = C.idle_bytes.find(device);
    return it == C.idle_bytes.end() ? 0 : it->second;
}

void dev_release_cached(int device) {
    DevCache &C = dev_cache();
    std::vector<std::pair<int, void *>> blocks;
    {
        std::lock_guard<std::mutex> g(C.mu);
        for (auto &d : C.idle) {
            if (device >= 0 && d.first != device) continue;
            for (auto &b : d.second) blocks.push_back({d.first, b.second});
            d.second.clear();
            C.idle_bytes[d.first] = 0;
        }
    }
    int cur = 0;
    cudaGetDevice(&cur);
    for (auto &b : blocks) {
        if (b.first != cur) cudaSetDevice(b.first);
        cudaFree(b.second);
        if (b.first != cur) cudaSetDevice(cur);
    }
}

size_t solver_layout(int n, int prec, int m, bool pc, unsigned char *base, SolverBufs *o, int n_rhs,
                     SolverBufs *extra, int krylov_copy) {
    size_t off = 0;
    auto take = [&](size_t bytes) -> void * {
        void *p = base ? (void *)(base + off) : nullptr;
        off += round_up(bytes, 256);
        return p;
    };
    const size_t N = (size_t)n, lda = round_up(N, 32);
    const size_t esz = prec == 0 ? 16 : 8;
    SolverBufs d;
    d.A = take(N * lda * esz);
    if (prec != 0 && n_rhs == 1 && (krylov_copy == 0 || krylov_copy == 2)) {
        d.A16 = take(N * lda * 4);
        d.rs = (float *)take(N * (size_t)mv_chunks(n) * 4);
    }
    if (prec != 0 && n_rhs == 1 && krylov_copy == 2) {
        const size_t nb = (size_t)blr_blocks(n), terms = nb * nb * kBlrMaxRank * kBlrB;
        d.blr_nb = (int)nb;
        d.blr_rank = (int *)take(nb * nb * 4);
        d.blr_U = (float2 *)take(terms * 8);
        d.blr_V = (float2 *)take(terms * 8);
        d.blr_U16 = (unsigned *)take(terms * 4);
        d.blr_V16 = (unsigned *)take(terms * 4);
        d.blr_scale = (float *)take(nb * nb * kBlrMaxRank * 4);
    }
    if (pc) {
        const size_t pb = precond_bytes(n, prec);
        d.Minv = take(prec == 0 ? pb / 2 : pb);
        if (prec == 0) d.Mwork = take(pb / 2);
    }
    d.status = (int *)take(16);
    d.ctr = (unsigned *)take(16);
    d.bct = (int *)take(N * 4);
    d.adm = (double *)take(2 * N * 8);
    auto per_rhs = [&](SolverBufs &q) {
        q.b = (double2 *)take(N * 16);
        q.x = (double2 *)take(N * 16);
        q.r = (double2 *)take(N * 16);
        // complex64 systems keep w and the Krylov basis in float pairs
        const size_t vsz = prec == 0 ? 16 : 8;
        q.w = (double2 *)take(N * vsz);
        q.z = (double2 *)take(N * 16);
        q.V = (double2 *)take((size_t)(m + 1) * N * vsz);
        q.mvp = (double2 *)take(mvp_elems(n) * 16);
        if (prec != 0) {   // complex64: float copies of the product's input
            q.xh = (float2 *)take(xsplit_elems(n) * 8);
            q.xf = (float4 *)take(xsplit_elems(n) * 16);
        }
        if (pc) {
            q.pcy = take(N * 16);
            q.pcz = take(N * 16);
        }
        q.dpa = (double2 *)take(dp_elems(n) * 16);
        q.dpb = (double2 *)take(dp_elems(n) * 16);
        q.nrmp = (double *)take((size_t)vec_blocks(n) * 8);
        q.H = (double2 *)take((size_t)(m + 1) * m * 16);
        q.cs = (double2 *)take((size_t)m * 16);
        q.sn = (double2 *)take((size_t)m * 16);
        q.g = (double2 *)take((size_t)(m + 1) * 16);
        q.y = (double2 *)take((size_t)m * 16);
        q.hsum = (double2 *)take((size_t)(m + 1) * 16);
        q.phi = (double *)take(N * 16);
        q.vel = (double *)take(4 * N * 16);
        q.phi32 = (float *)take(N * 8);
        q.vel32 = (float *)take(4 * N * 8);
        q.ivi = (int *)take(N * 4);
        q.cols = (int *)take(N * 4);
        q.bcv = (double *)take(8 * N * 8);
        q.src = (double *)take(5 * (size_t)kInlineSources * 8);
    };
    per_rhs(d);
    for (int r = 1; r < n_rhs; ++r) {
        SolverBufs q = d;   // shared fields
        per_rhs(q);
        if (extra) extra[r - 1] = q;
    }
    if (o) *o = d;
    return off;
}

}  // namespace bem


namespace {

// host copy of a device buffer
bem_status fetch(cudaStream_t st, const void *dsrc, void *hdst, size_t bytes) {
    CU(cudaMemcpyAsync(hdst, dsrc, bytes, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    return BEM_OK;
}

const char *subdivision_message(int code) {
    return code == 1 ? "number of subelements which are subdivided in a loop must <= 15"
                     : "number of subelements must be < 220";
}

}  // namespace

namespace bem {

// Frequency data into the solver's block (internal element order).  NumCalc
// does the same per frequency in NC_UpdateFreqCurves before assembly.
bem_status upload_freq(bem_solver_t s, const bem_frequency_desc *f, cudaStream_t st, int rhs) {
    const int n = s->n;
    if (rhs < 0 || rhs >= s->n_rhs) return fail(BEM_ERR_INVALID, "right-hand side %d of %d", rhs, s->n_rhs);
    const SolverBufs &B = s->buf(rhs);
    if (!(f->wave_number > 0.0)) return fail(BEM_ERR_INVALID, "wave number must be > 0");
    if (f->n_point < 0 || f->n_plane < 0) return fail(BEM_ERR_INVALID, "negative source count");
    if ((f->n_point && (!f->point_xyz || !f->point_amp)) || (f->n_plane && (!f->plane_dir || !f->plane_amp)))
        return fail(BEM_ERR_INVALID, "source arrays missing");
    bem::DevFreq &F = rhs == 0 ? s->freq : s->xfreq[rhs - 1];
    F = bem::DevFreq{};
    const double htf = f->time_factor == -1.0 ? -1.0 : 1.0;
    const double tao = f->tao == -1.0 ? -1.0 : 1.0;
    F.k = f->wave_number;
    F.wr = htf * f->wave_number;
    F.tao = tao;
    F.beta_im = tao < 0 ? 0.0 : htf / f->wave_number;   // NC_EquationSystem.cpp:85-86
    F.kf = (float)F.k;
    F.wrf = (float)F.wr;
    F.taof = (float)F.tao;
    F.beta_imf = (float)F.beta_im;
    const std::vector<int> &ext = s->mesh->ext_of_int;
    std::vector<int> cols, bct;
    std::vector<double> bcv, adm, src;
    if (rhs > 0) {   // the matrix data of right-hand side 0
        F.bc_type = s->freq.bc_type;
        F.adm = s->freq.adm;
    }
    if (f->bc_type && rhs == 0) {
        for (int j = 0; j < n; ++j)
            if (f->bc_type[j] < 0 || f->bc_type[j] > 2)
                return fail(BEM_ERR_INVALID, "element %d: boundary condition type %d unsupported", j, f->bc_type[j]);
        bct.resize(n);
        for (int i = 0; i < n; ++i) bct[i] = f->bc_type[ext[i]];
        CU(cudaMemcpyAsync(B.bct, bct.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st));
        F.bc_type = B.bct;
    }
    if (f->bc_value) {
        bcv.assign(8 * (size_t)n, 0.0);
        for (int i = 0; i < n; ++i) {
            const int j = ext[i];
            bool nz = false;
            for (int a = 0; a < 4; ++a) {
                const double re = f->bc_value[8 * (size_t)j + 2 * a], im = f->bc_value[8 * (size_t)j + 2 * a + 1];
                bcv[2 * ((size_t)a * n + i)] = re;
                bcv[2 * ((size_t)a * n + i) + 1] = im;
                // NumCalc's test: |value| > EPSY on the element's nodes (NC_EquationSystem.cpp:264-275)
                if (a < s->mesh->nvert[i] && std::sqrt(re * re + im * im) > 1.0e-14) nz = true;
            }
            if (nz) cols.push_back(i);
        }
        CU(cudaMemcpyAsync(B.bcv, bcv.data(), sizeof(double) * bcv.size(), cudaMemcpyHostToDevice, st));
        F.bc_val = B.bcv;
    }
    if (f->admittance && rhs == 0) {
        adm.resize(2 * (size_t)n);
        for (int i = 0; i < n; ++i) {
            adm[2 * (size_t)i] = f->admittance[2 * (size_t)ext[i]];
            adm[2 * (size_t)i + 1] = f->admittance[2 * (size_t)ext[i] + 1];
        }
        CU(cudaMemcpyAsync(B.adm, adm.data(), sizeof(double) * adm.size(), cudaMemcpyHostToDevice, st));
        F.adm = B.adm;
    }
    if (!cols.empty()) {
        CU(cudaMemcpyAsync(B.cols, cols.data(), sizeof(int) * cols.size(), cudaMemcpyHostToDevice, st));
        F.bc_cols = B.cols;
        F.n_bc_cols = (int)cols.size();
    }
    const size_t nsrc = 5 * (size_t)f->n_point + 5 * (size_t)f->n_plane;
    if (nsrc) {
        // complex amplitudes first so that they start on 16-byte boundaries
        // (the kernels read them as double2), coordinates after them
        src.reserve(nsrc);
        for (int i = 0; i < 2 * f->n_point; ++i) src.push_back(f->point_amp[i]);
        for (int i = 0; i < 2 * f->n_plane; ++i) src.push_back(f->plane_amp[i]);
        for (int i = 0; i < 3 * f->n_point; ++i) src.push_back(f->point_xyz[i]);
        for (int i = 0; i < 3 * f->n_plane; ++i) src.push_back(f->plane_dir[i]);
        double *dst = B.src;
        if (f->n_point + f->n_plane > bem::kInlineSources) {
            if (rhs > 0) return fail(BEM_ERR_INVALID, "more than %d sources on right-hand side %d", bem::kInlineSources, rhs);
            CU(cudaStreamSynchronize(st));
            bem::dev_free(s->src_extra);
            s->src_extra = nullptr;
            CU(dalloc(&s->src_extra, src.size()));
            dst = s->src_extra;
        }
        CU(cudaMemcpyAsync(dst, src.data(), sizeof(double) * src.size(), cudaMemcpyHostToDevice, st));
        F.n_point = f->n_point;
        F.n_plane = f->n_plane;
        F.ps_amp = dst;
        F.pw_amp = dst + 2 * (size_t)f->n_point;
        F.ps_xyz = dst + 2 * (size_t)f->n_point + 2 * (size_t)f->n_plane;
        F.pw_dir = F.ps_xyz + 3 * (size_t)f->n_point;
    }
    // the host vectors above go out of scope: finish the copies
    CU(cudaStreamSynchronize(st));
    return BEM_OK;
}

bem_status map_result(const KState &q) {
    switch (q.result) {
    case bem::kResConverged: return BEM_OK;
    case bem::kResBreakdown:
        if (q.cycles == 0) return fail(BEM_ERR_INVALID, "right-hand side is not finite");
        return fail(BEM_ERR_NOT_CONVERGED, "GMRES breakdown (non-finite residual)");
    case bem::kResStagnated:
        return fail(BEM_ERR_NOT_CONVERGED, "iterative refinement stagnated at relative residual %.3e after %d iterations",
                    q.rel, q.iters);
    default:
        return fail(BEM_ERR_NOT_CONVERGED, "GMRES reached %d iterations, relative residual %.3e", q.iters, q.rel);
    }
}

}  // namespace bem

namespace {

// One stream and one Krylov engine per thread and precision for the batched
// entry points.
struct BatchCtx {
    cudaStream_t st = nullptr;
    cudaEvent_t ev[6] = {};
    std::unique_ptr<bem::Engine> eng[2];
    unsigned *ctr = nullptr;
    ~BatchCtx() {
        for (auto &e : eng) e.reset();
        cudaFree(ctr);
        for (auto &e : ev)
            if (e) cudaEventDestroy(e);
        if (st) cudaStreamDestroy(st);
    }
};
thread_local std::unique_ptr<BatchCtx> t_batch;

bem_status batch_ctx(BatchCtx **out) {
    if (!t_batch) {
        auto c = std::make_unique<BatchCtx>();
        CU(cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking));
        for (auto &e : c->ev) CU(cudaEventCreate(&e));
        CU(cudaMalloc(&c->ctr, 4 * sizeof(unsigned)));
        CU(cudaMemset(c->ctr, 0, 4 * sizeof(unsigned)));
        t_batch = std::move(c);
    }
    *out = t_batch.get();
    return BEM_OK;
}

}  // namespace

namespace bem {

// ---- group operations shared by the single-solver and batched entry points

// The assembly's launch shape for a group: the tuned choice for its largest
// system.  On the first assembly of an untuned key every candidate shape
// assembles the group once (each run writes the same bits), timed with CUDA
// events, and the fastest is kept.
bem_status tuned_asm_shape(bem_solver_t *ss, int cnt, cudaStream_t st, unsigned *ctr, bem::AsmShape *out) {
    const int prec = ss[0]->prec;
    int big = 0;
    for (int i = 1; i < cnt; ++i)
        if (ss[i]->n > ss[big]->n) big = i;
    const bem::TuneChoice tc = bem::tune_lookup(ss[big]->n, prec, ss[big]->n_rhs);
    *out = tc.asm_shape;
    if (!bem::tune_enabled() || tc.asm_tuned) return BEM_OK;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    for (auto &e : ev) CU(cudaEventCreate(&e));
    std::unique_ptr<bem::AsmBatch> t(new bem::AsmBatch());
    float best = 1e30f;
    bem::AsmShape pick = tc.asm_shape;
    cudaError_t err = cudaSuccess;
    // the default shape first; when one assembly of the group takes longer
    // than kTuneAsmMaxMs (large FP64 systems) the default is kept without
    // running the other candidates
    constexpr float kTuneAsmMaxMs = 100.f;
    std::vector<bem::AsmShape> cand(1, bem::AsmShape());
    for (int fa = 1; fa <= bem::kFarPerSmMax; ++fa)
        for (int ne = 1; ne <= 2; ++ne) {
            bem::AsmShape sh;
            sh.far_per_sm = fa;
            sh.near_per_sm = ne;
            if (sh.far_per_sm != cand[0].far_per_sm || sh.near_per_sm != cand[0].near_per_sm) cand.push_back(sh);
        }
    for (size_t ci = 0; ci < cand.size() && err == cudaSuccess; ++ci) {
        {
            const bem::AsmShape sh = cand[ci];
            err = cudaEventRecord(ev[0], st);
            for (int c0 = 0; c0 < cnt && err == cudaSuccess; c0 += bem::kMaxAsm) {
                const int k = std::min(bem::kMaxAsm, cnt - c0);
                t->B = k;
                for (int i = 0; i < k; ++i) t->sys[i] = ss[c0 + i]->asys();
                bem::asm_batch_finish(*t);
                err = bem::launch_assemble(*t, prec, ctr, st, sh);
            }
            if (err == cudaSuccess) err = cudaEventRecord(ev[1], st);
            if (err == cudaSuccess) err = cudaEventSynchronize(ev[1]);
            float ms = 0.f;
            if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, ev[0], ev[1]);
            if (err == cudaSuccess && ms < best) {
                best = ms;
                pick = sh;
            }
            if (ci == 0 && ms > kTuneAsmMaxMs) break;
        }
    }
    for (auto &e : ev) cudaEventDestroy(e);
    CU(err);
    bem::tune_store_asm(ss[big]->n, prec, ss[big]->n_rhs, pick, best);
    *out = pick;
    return BEM_OK;
}

bem_status assemble_group(bem_solver_t *ss, int cnt, cudaStream_t st, unsigned *ctr, cudaEvent_t e0,
                          cudaEvent_t e1, bem_status *rcs) {
    const int prec = ss[0]->prec;
    for (int i = 0; i < cnt; ++i) CU(cudaMemsetAsync(ss[i]->d.status, 0, sizeof(int), st));
    bem::AsmShape shape;
    bem_status trc = tuned_asm_shape(ss, cnt, st, ctr, &shape);
    if (trc != BEM_OK) return trc;
    CU(cudaEventRecord(e0, st));
    std::unique_ptr<bem::AsmBatch> t(new bem::AsmBatch());
    for (int c0 = 0; c0 < cnt; c0 += bem::kMaxAsm) {
        const int k = std::min(bem::kMaxAsm, cnt - c0);
        t->B = k;
        for (int i = 0; i < k; ++i) t->sys[i] = ss[c0 + i]->asys();
        bem::asm_batch_finish(*t);
        CU(bem::launch_assemble(*t, prec, ctr, st, shape));
        CU(bem::launch_rhs(*t, st));
    }
    CU(cudaEventRecord(e1, st));
    std::vector<int> code(cnt, 0);
    for (int i = 0; i < cnt; ++i)
        CU(cudaMemcpyAsync(&code[i], ss[i]->d.status, sizeof(int), cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    float ms = 0.f;
    CU(cudaEventElapsedTime(&ms, e0, e1));
    bem_status first = BEM_OK;
    for (int i = 0; i < cnt; ++i) {
        bem_solver_t s = ss[i];
        s->info.assemble_ms = ms;
        s->info.n_near_pairs = (int64_t)(s->mesh->n_near - s->n);   // subdivided pairs (self pairs excluded)
        s->have_freq = true;
        s->factored = false;
        s->solved = false;
        rcs[i] = BEM_OK;
        if (code[i] != 0) {
            rcs[i] = fail(BEM_ERR_SUBDIVISION, "%s", subdivision_message(code[i]));
            if (first == BEM_OK) first = rcs[i];
        }
    }
    return first;
}

// Block low-rank copies (BlrBatch) and fp16 copies (SplitBatch; for a
// solver with a block low-rank copy only the segments that copy reads) of
// the complex64 matrices that have them.
cudaError_t split_group(bem_solver_t *ss, int cnt, cudaStream_t st) {
    // the block low-rank copies first: their ranks say which fp16 segments
    // are read
    std::unique_ptr<bem::BlrBatch> bt(new bem::BlrBatch());
    bt->B = 0;
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < cnt && e == cudaSuccess; ++i) {
        const bem::SolverBufs &d = ss[i]->d;
        if (d.blr_nb <= 0) continue;
        bem::BlrSys &q = bt->sys[bt->B++];
        q.A = d.A;
        q.lda = ss[i]->lda;
        q.n = ss[i]->n;
        q.rank = d.blr_rank;
        q.U = d.blr_U;
        q.V = d.blr_V;
        q.U16 = d.blr_U16;
        q.V16 = d.blr_V16;
        q.scale = d.blr_scale;
        if (bt->B == bem::kMaxAsm) {
            bem::blr_batch_finish(*bt);
            e = bem::launch_blr_compress(*bt, st);
            bt->B = 0;
        }
    }
    if (e == cudaSuccess && bt->B > 0) {
        bem::blr_batch_finish(*bt);
        e = bem::launch_blr_compress(*bt, st);
    }
    std::unique_ptr<bem::SplitBatch> t(new bem::SplitBatch());
    t->B = 0;
    for (int i = 0; i < cnt && e == cudaSuccess; ++i) {
        const bem::SolverBufs &d = ss[i]->d;
        if (!d.A16) continue;
        bem::SplitSys &q = t->sys[t->B++];
        q.A = d.A;
        q.lda = ss[i]->lda;
        q.n = ss[i]->n;
        q.A16 = d.A16;
        q.rs = d.rs;
        q.blr_rank = d.blr_nb > 0 ? d.blr_rank : nullptr;
        q.blr_nb = d.blr_nb;
        if (t->B == bem::kMaxAsm) {
            bem::split_batch_finish(*t);
            e = bem::launch_split16(*t, st);
            t->B = 0;
        }
    }
    if (e == cudaSuccess && t->B > 0) {
        bem::split_batch_finish(*t);
        e = bem::launch_split16(*t, st);
    }
    return e;
}

// A second stream per device for the preconditioner's set-up, so that the
// block inverses (latency bound: a barrier per pivot) run beside the Krylov
// copies (bound by DRAM traffic); both only read A.  nullptr if it cannot be
// had (then everything runs on the caller's stream).
cudaStream_t aux_stream(cudaStream_t st) {
    static std::mutex mu;
    static cudaStream_t streams[64] = {};
    int dev = -1, sdev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    if (cudaStreamGetDevice(st, &sdev) != cudaSuccess || sdev != dev) {
        cudaGetLastError();
        return nullptr;
    }
    std::lock_guard<std::mutex> lk(mu);
    if (!streams[dev] && cudaStreamCreateWithFlags(&streams[dev], cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        streams[dev] = nullptr;
    }
    return streams[dev];
}

bem_status precond_group(bem_solver_t *ss, int cnt, cudaStream_t st) {
    const int prec = ss[0]->prec;
    std::unique_ptr<bem::PcBatch> pt(new bem::PcBatch());
    std::vector<bem_solver_t> pcs;
    for (int i = 0; i < cnt; ++i) {
        ss[i]->have_precond = false;
        if (ss[i]->precond) pcs.push_back(ss[i]);
        CU(cudaMemsetAsync(ss[i]->d.x, 0, sizeof(double2) * ss[i]->n, st));
    }
    // the inverses on the second stream, from the assembled A
    cudaStream_t ps = st;
    struct Events {
        cudaEvent_t e[2] = {nullptr, nullptr};
        ~Events() {
            for (cudaEvent_t x : e)
                if (x) cudaEventDestroy(x);
        }
    } evs;
    cudaEvent_t *ev = evs.e;
    cudaStream_t aux = pcs.empty() ? nullptr : aux_stream(st);
    if (aux && cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming) == cudaSuccess &&
        cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming) == cudaSuccess) {
        CU(cudaEventRecord(ev[0], st));
        CU(cudaStreamWaitEvent(aux, ev[0], 0));
        ps = aux;
    } else {
        cudaGetLastError();
    }
    std::vector<bem_solver_t> bj;   // block-Jacobi; the scaling ones are set here
    for (bem_solver_t s : pcs) {
        if (!s->pc_scaling) {
            bj.push_back(s);
            continue;
        }
        CU(cudaMemsetAsync(s->d.status, 0, sizeof(int), ps));
        CU(bem::launch_pc_scaling(s->psys(), prec, ps));
    }
    for (size_t c0 = 0; c0 < bj.size(); c0 += bem::kMaxAsm) {
        const int k = (int)std::min<size_t>(bem::kMaxAsm, bj.size() - c0);
        pt->B = k;
        for (int i = 0; i < k; ++i) {
            CU(cudaMemsetAsync(bj[c0 + i]->d.status, 0, sizeof(int), ps));
            pt->sys[i] = bj[c0 + i]->psys();
        }
        bem::pc_batch_finish(*pt);
        CU(bem::launch_block_inverse(*pt, prec, ps));
    }
    if (ps != st) CU(cudaEventRecord(ev[1], ps));
    // the Krylov copies on the caller's stream meanwhile
    const cudaError_t se = split_group(ss, cnt, st);
    if (ps != st) CU(cudaStreamWaitEvent(st, ev[1], 0));
    CU(se);
    if (!pcs.empty()) {
        std::vector<int> sing(pcs.size(), 0);
        for (size_t i = 0; i < pcs.size(); ++i)
            CU(cudaMemcpyAsync(&sing[i], pcs[i]->d.status, sizeof(int), cudaMemcpyDeviceToHost, st));
        CU(cudaStreamSynchronize(st));
        for (size_t i = 0; i < pcs.size(); ++i) pcs[i]->have_precond = sing[i] == 0;   // singular block: no M
    }
    return BEM_OK;
}

// Restarted GMRES of every solver in ss on the engine: preconditioner set-up,
// then iteration bodies until every system has finished.
// The complex64 product's strip height of every solver in ss: the tuned
// choice of its key; on the first solve of an untuned key every candidate
// height times one product of that system (the products write only scratch
// partials, and every height gives the same partials).
bem_status tuned_strips(bem_solver_t *ss, int cnt, bem::Engine *eng) {
    for (int i = 0; i < cnt; ++i) {
        bem_solver_t s = ss[i];
        if (s->prec != BEM_PREC_MIXED || s->n_rhs > 1) continue;   // grouped products have fixed strips
        const bem::TuneChoice tc = bem::tune_lookup(s->n, s->prec, 1);
        s->mv_strip = tc.mv_strip;
        if (!bem::tune_enabled() || tc.mv_tuned) continue;
        static const int kCand[4] = {16, 32, 64, 128};
        float best = 1e30f;
        int pick = tc.mv_strip;
        for (int c : kCand) {
            s->mv_strip = c;
            float ms = 0.f;
            bem::KSys k = s->ksys();
            if (k.blr_nb > 0) k.A16 = nullptr;   // its fp16 copy is partial: time the residual product
            const cudaError_t e = eng->time_product(k, &ms);
            if (e == cudaErrorLaunchTimeout)
                return fail(BEM_ERR_DEVICE_TIMEOUT, "matrix-vector product: a bounded device wait gave up");
            CU(e);
            if (ms < best) {
                best = ms;
                pick = c;
            }
        }
        bem::tune_store_mv(s->n, s->prec, 1, pick, best);
        for (int j = i; j < cnt; ++j)   // the same key further on
            if (ss[j]->prec == s->prec && ss[j]->n_rhs <= 1 && bem::tune_bucket(ss[j]->n) == bem::tune_bucket(s->n))
                ss[j]->mv_strip = pick;
    }
    return BEM_OK;
}

bem_status solve_group(bem_solver_t *ss, int cnt, bem::Engine *eng, cudaStream_t st, cudaEvent_t e0,
                       cudaEvent_t e1, bem_status *rcs) {
    CU(cudaEventRecord(e0, st));
    bem_status prc = precond_group(ss, cnt, st);
    if (prc != BEM_OK) return prc;
    prc = tuned_strips(ss, cnt, eng);
    if (prc != BEM_OK) return prc;
    bem_status first = BEM_OK;
    for (int c0 = 0; c0 < cnt; c0 += bem::kMaxSys) {
        const int k = std::min(bem::kMaxSys, cnt - c0);
        std::vector<bem::KSys> sys(k);
        std::vector<bem::KState> init(k);
        long long guard = 0;
        for (int i = 0; i < k; ++i) {
            sys[i] = ss[c0 + i]->ksys();
            init[i] = ss[c0 + i]->kinit();
            guard = std::max<long long>(guard, 2LL * ss[c0 + i]->max_iter + 64);
        }
        CU(eng->set_batch(sys, init));
        bool all_done = false;
        for (long long body = 0; body < guard && !all_done; ++body) {
            const cudaError_t be = eng->run_body();
            if (be == cudaErrorLaunchTimeout)
                return fail(BEM_ERR_DEVICE_TIMEOUT, "matrix-vector product: a bounded device wait gave up");
            CU(be);
            all_done = true;
            for (int i = 0; i < k; ++i)
                if (eng->states()[i].phase != bem::kPhaseFinished) all_done = false;
        }
        CU(cudaEventRecord(e1, st));
        CU(cudaEventSynchronize(e1));
        float ms = 0.f;
        CU(cudaEventElapsedTime(&ms, e0, e1));
        for (int i = 0; i < k; ++i) {
            bem_solver_t s = ss[c0 + i];
            const bem::KState &q = eng->states()[i];
            s->info.solve_ms = ms;
            s->info.iterations = q.iters;
            s->info.restarts = q.cycles;
            s->info.rel_residual = q.rel;
            s->info.matvec_ms = eng->timing_ok() ? eng->matvec_ms() : 0.0;
            s->info.n_matvec = q.n_mv;
            s->solved = true;
            if (q.phase != bem::kPhaseFinished) rcs[c0 + i] = fail(BEM_ERR_DEVICE_TIMEOUT, "GMRES did not finish");
            else rcs[c0 + i] = map_result(q);
            if (rcs[c0 + i] != BEM_OK && first == BEM_OK) first = rcs[c0 + i];
        }
        CU(cudaEventRecord(e0, st));
    }
    return first;
}

// Point buffers for n_pts points: the points, and potentials and gradients
// for each of the solver's right-hand sides.
bem_status ensure_points(bem_solver_t s, int n_pts) {
    if (n_pts <= s->pts_cap) return BEM_OK;
    CU(cudaStreamSynchronize(s->st));
    bem::dev_free(s->pts); bem::dev_free(s->pot); bem::dev_free(s->grad);
    s->pts = s->pot = s->grad = nullptr;
    s->pts_cap = 0;
    CU(dalloc(&s->pts, 3 * (size_t)n_pts));
    CU(dalloc(&s->pot, 2 * (size_t)n_pts * s->n_rhs));
    CU(dalloc(&s->grad, 6 * (size_t)n_pts * s->n_rhs));
    s->pts_cap = n_pts;
    return BEM_OK;
}

// Fields and projection of every solver in ss; pts[i] (host) may be null
// when npts[i] == 0.
bem_status project_group(bem_solver_t *ss, int cnt, const int32_t *npts, const double *const *pts,
                         double *const *pot_out, double *const *grad_out, cudaStream_t st, cudaEvent_t e0,
                         cudaEvent_t e1, bem_status *rcs) {
    const int prec = ss[0]->prec;
    for (int i = 0; i < cnt; ++i) {
        const int np = npts ? npts[i] : 0;
        bem_status rc = ensure_points(ss[i], np);
        if (rc != BEM_OK) return rc;
        if (np > 0) CU(cudaMemcpyAsync(ss[i]->pts, pts[i], sizeof(double) * 3 * np, cudaMemcpyHostToDevice, st));
        CU(cudaMemsetAsync(ss[i]->d.status, 0, sizeof(int), st));
    }
    CU(cudaEventRecord(e0, st));
    std::unique_ptr<bem::ProjBatch> t(new bem::ProjBatch());
    for (int c0 = 0; c0 < cnt; c0 += bem::kMaxAsm) {
        const int k = std::min(bem::kMaxAsm, cnt - c0);
        t->B = k;
        for (int i = 0; i < k; ++i) {
            bem_solver_t s = ss[c0 + i];
            const int np = npts ? npts[c0 + i] : 0;
            t->sys[i] = s->prsys(np, s->pts, (double *)s->pot, (double *)s->grad);
        }
        bem::proj_batch_finish(*t);
        CU(bem::launch_fields(*t, st));
        CU(bem::launch_project(*t, prec, st));
    }
    CU(cudaEventRecord(e1, st));
    std::vector<int> code(cnt, 0);
    for (int i = 0; i < cnt; ++i) {
        const int np = npts ? npts[i] : 0;
        if (np > 0 && pot_out && pot_out[i])
            CU(cudaMemcpyAsync(pot_out[i], ss[i]->pot, sizeof(double) * 2 * np, cudaMemcpyDeviceToHost, st));
        if (np > 0 && grad_out && grad_out[i])
            CU(cudaMemcpyAsync(grad_out[i], ss[i]->grad, sizeof(double) * 6 * np, cudaMemcpyDeviceToHost, st));
        CU(cudaMemcpyAsync(&code[i], ss[i]->d.status, sizeof(int), cudaMemcpyDeviceToHost, st));
    }
    CU(cudaStreamSynchronize(st));
    float ms = 0.f;
    CU(cudaEventElapsedTime(&ms, e0, e1));
    bem_status first = BEM_OK;
    for (int i = 0; i < cnt; ++i) {
        ss[i]->info.project_ms = ms;
        rcs[i] = BEM_OK;
        if (code[i] != 0) {
            rcs[i] = fail(BEM_ERR_SUBDIVISION, "evaluation point too close to the boundary: subdivision limit");
            if (first == BEM_OK) first = rcs[i];
        }
    }
    return first;
}

bem_status solution_to_host(bem_solver_t s, cudaStream_t st, double *x_host, int rhs) {
    std::vector<double> t(2 * (size_t)s->n);
    bem_status rc = fetch(st, s->buf(rhs).x, t.data(), t.size() * sizeof(double));
    if (rc != BEM_OK) return rc;
    const std::vector<int> &ext = s->mesh->ext_of_int;
    for (int i = 0; i < s->n; ++i) {
        x_host[2 * (size_t)ext[i]] = t[2 * (size_t)i];
        x_host[2 * (size_t)ext[i] + 1] = t[2 * (size_t)i + 1];
    }
    return BEM_OK;
}

bem::Engine *solver_engine(bem_solver_t s) {
    if (!s->eng) s->eng.reset(new bem::Engine(s->prec == BEM_PREC_FP64 ? 0 : 1, s->st));
    return s->eng.get();
}

}  // namespace bem

using bem::assemble_group;
using bem::ensure_points;
using bem::map_result;
using bem::precond_group;
using bem::project_group;
using bem::solution_to_host;
using bem::solve_group;
using bem::solver_engine;
using bem::upload_freq;

extern "C" {

const char *bem_last_error(void) { return g_err.c_str(); }

const char *bem_version(void) { return "mesh2hrtf_gb300 1.1 (sm_103a)"; }

int64_t bem_kernel_launches(void) { return (int64_t)bem::launches(); }

bem_status bem_set_device(int32_t device) {
    CU(cudaSetDevice(device));
    return ensure_device_init();
}

double bem_footprint_bytes(int32_t n_elem, int32_t precision, int32_t restart) {
    return bem_footprint_multi(n_elem, precision, restart, 1);
}

double bem_footprint_multi(int32_t n_elem, int32_t precision, int32_t restart, int32_t n_rhs) {
    const int m = restart > 0 ? restart : 60;
    const int prec = precision == BEM_PREC_FP64 ? 0 : 1;
    return (double)bem::solver_layout(std::max(n_elem, 1), prec, m, true, nullptr, nullptr, std::max(n_rhs, 1));
}

double bem_mesh_footprint_bytes(int32_t n_elem, int32_t n_sym_planes) {
    const int n = std::max(n_elem, 1);
    const int nref = 1 << std::min(std::max(n_sym_planes, 0), 3);
    // element tables: 1 + 12 + 3 + 3 + 1 + 1 words of 8 B, 3 + 3 + 10 + 12 + 1 + 3 + 12 of 4 B
    const double tables = (double)n * (4.0 + 20.0 * 8.0 + 44.0 * 4.0);
    const double near = (double)n * nref * 48.0 * sizeof(int2);   // the list's first allocation
    return tables + (double)bem::image_table_bytes(n, nref) + near;
}

bem_status bem_release_cached_memory(void) {
    bem::dev_release_cached(-1);
    return BEM_OK;
}

bem_status bem_device_memory(int32_t device, double *free_bytes, double *total_bytes) {
    if (!free_bytes || !total_bytes) return fail(BEM_ERR_INVALID, "null argument");
    int cur = 0;
    CU(cudaGetDevice(&cur));
    CU(cudaSetDevice(device));
    size_t fr = 0, tot = 0;
    const cudaError_t e = cudaMemGetInfo(&fr, &tot);
    cudaSetDevice(cur);
    if (e != cudaSuccess) return fail(BEM_ERR_CUDA, "cudaMemGetInfo: %s", cudaGetErrorString(e));
    *free_bytes = (double)fr + (double)bem::dev_cached_bytes(device);
    *total_bytes = (double)tot;
    return BEM_OK;
}

bem_status bem_mesh_create(const bem_mesh_desc *d, bem_mesh_t *out) {
    if (!d || !out) return fail(BEM_ERR_INVALID, "null argument");
    *out = nullptr;
    if (d->n_elem <= 0 || d->n_nodes <= 0 || !d->nodes || !d->conn || !d->nvert)
        return fail(BEM_ERR_INVALID, "mesh needs elements, nodes, connectivity and vertex counts");
    if (d->n_elem > bem::kMaxElements)
        return fail(BEM_ERR_INVALID, "%d elements: at most %d", d->n_elem, bem::kMaxElements);
    // symmetry planes: NC.inp codes -> images (NC_Input.cpp:342-343,470-491)
    bem::DevSym sym{};
    int sign[3] = {0, 0, 0}, nplanes = 0;
    for (int k = 0; k < 3; ++k) {
        const int c = d->sym_planes[k];
        if (c < 0 || c > 4) return fail(BEM_ERR_INVALID, "symmetry code %d on axis %d (0 .. 4 allowed)", c, k);
        sym.coord[k] = d->sym_coords[k];
        if (c) {
            sign[k] = (c == 2 || c == 4) ? -1 : 1;
            sym.axes |= 1u << k;
            ++nplanes;
        }
    }
    sym.nref = 1 << nplanes;
    {
        // axis of each reflection step, NC_ReflectPointVector (NC_3dFunctions.cpp:190-228)
        static const int nrefdi[8] = {0, 0, 1, 0, 2, 0, 1, 0};
        int first_free = 0, first_plane = 0;
        for (int k = 2; k >= 0; --k) {
            if (!sign[k]) first_free = k + 1;
            else first_plane = k;
        }
        int rf = 1;
        for (int kref = 1; kref < sym.nref; ++kref) {
            int dir = 0;
            if (sym.nref == 8) dir = nrefdi[kref];
            else if (sym.nref == 4) {
                dir = first_free + nrefdi[kref];
                if (dir >= 3) dir -= 3;
            } else dir = first_plane;
            sym.rdir[kref] = (unsigned char)dir;
            if (sign[dir] < 0) rf = -rf;
            if (rf < 0) sym.rneg |= 1u << kref;
        }
    }
    bem_status s = ensure_device_init();
    if (s != BEM_OK) return s;
    const int n = d->n_elem;
    // geometry per element in the caller's order
    std::vector<double> P(12 * (size_t)n, 0.0), C(3 * (size_t)n), NR(3 * (size_t)n), AR(n);
    std::vector<int> nvx(n);
    for (int j = 0; j < n; ++j) {
        const int nv = d->nvert[j];
        if (nv != 3 && nv != 4) return fail(BEM_ERR_INVALID, "element %d has %d vertices (3 or 4 allowed)", j, nv);
        nvx[j] = nv;
        double p[4][3] = {{0}};
        for (int a = 0; a < nv; ++a) {
            const int node = d->conn[4 * (size_t)j + a];
            if (node < 0 || node >= d->n_nodes) return fail(BEM_ERR_INVALID, "element %d: node index %d", j, node);
            for (int k = 0; k < 3; ++k) p[a][k] = P[12 * (size_t)j + 3 * a + k] = d->nodes[3 * (size_t)node + k];
        }
        double c[3], nr[3], ar;
        element_geometry(nv, p, c, nr, &ar);
        if (d->centers) for (int k = 0; k < 3; ++k) c[k] = d->centers[3 * (size_t)j + k];
        if (d->normals) for (int k = 0; k < 3; ++k) nr[k] = d->normals[3 * (size_t)j + k];
        if (d->areas) ar = d->areas[j];
        if (!(ar > 0.0)) return fail(BEM_ERR_INVALID, "element %d has area %g", j, ar);
        for (int k = 0; k < 3; ++k) { C[3 * (size_t)j + k] = c[k]; NR[3 * (size_t)j + k] = nr[k]; }
        AR[j] = ar;
    }
    if (nplanes) {
        // all boundary nodes on one side of every plane, within a hundredth of
        // the mean element size (NC_Input.cpp:660-699)
        double asum = 0.0;
        for (int j = 0; j < n; ++j) asum += AR[j];
        const double dtl = std::sqrt(asum / n) / 100.0;
        for (int k = 0; k < 3; ++k) {
            if (!sign[k]) continue;
            double hi = -9.9e20, lo = 9.9e20;
            for (int j = 0; j < n; ++j)
                for (int a = 0; a < nvx[j]; ++a) {
                    const double v = P[12 * (size_t)j + 3 * a + k];
                    hi = std::max(hi, v);
                    lo = std::min(lo, v);
                }
            const double c = sym.coord[k];
            if (!((hi >= c - dtl && lo >= c - dtl) || (hi <= c + dtl && lo <= c + dtl)))
                return fail(BEM_ERR_INVALID, "All BE nodes must be located on the same side of a symmetric plane! "
                            "(axis %d)", k);
        }
    }
    // internal numbering along a Morton curve of the centres: consecutive
    // unknowns are neighbours, so the diagonal blocks of A carry the near
    // field (block-Jacobi preconditioner) and near pairs cluster per tile
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int j = 0; j < n; ++j)
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], C[3 * (size_t)j + k]);
            hi[k] = std::max(hi[k], C[3 * (size_t)j + k]);
        }
    std::vector<uint64_t> key(n);
    for (int j = 0; j < n; ++j) {
        uint64_t q[3];
        for (int k = 0; k < 3; ++k) {
            const double span = hi[k] - lo[k];
            const double u = span > 0 ? (C[3 * (size_t)j + k] - lo[k]) / span : 0.0;
            q[k] = (uint64_t)std::min(2097151.0, std::max(0.0, u * 2097151.0));
        }
        key[j] = spread3(q[0]) | spread3(q[1]) << 1 | spread3(q[2]) << 2;
    }
    std::vector<int> order(n);
    for (int j = 0; j < n; ++j) order[j] = j;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return key[a] < key[b]; });
    std::vector<double> v64(12 * (size_t)n, 0.0), c64(3 * (size_t)n), n64(3 * (size_t)n), area(n), sqa(n);
    std::vector<float> chi(3 * (size_t)n), clo(3 * (size_t)n), t32(10 * (size_t)n, 0.f), q32(12 * (size_t)n, 0.f),
        isqa(n), n32(3 * (size_t)n);
    std::vector<int> nvert(n), int_of_ext(n);
    for (int i = 0; i < n; ++i) {
        const int j = order[i];
        int_of_ext[j] = i;
        const int nv = nvx[j];
        nvert[i] = nv;
        double p[4][3] = {{0}};
        for (int a = 0; a < nv; ++a)
            for (int k = 0; k < 3; ++k) {
                p[a][k] = P[12 * (size_t)j + 3 * a + k];
                v64[(3 * a + k) * (size_t)n + i] = p[a][k];
            }
        const double *c = &C[3 * (size_t)j], *nr = &NR[3 * (size_t)j];
        const double ar = AR[j];
        for (int k = 0; k < 3; ++k) {
            c64[k * (size_t)n + i] = c[k];
            n64[k * (size_t)n + i] = nr[k];
            n32[k * (size_t)n + i] = (float)nr[k];
            const float h = (float)c[k];
            chi[k * (size_t)n + i] = h;
            clo[k * (size_t)n + i] = (float)(c[k] - (double)h);
        }
        area[i] = ar;
        sqa[i] = std::sqrt(ar);
        isqa[i] = (float)(1.0 / sqa[i]);
        if (nv == 3) {
            for (int k = 0; k < 3; ++k) {
                t32[k * (size_t)n + i] = (float)(p[0][k] - p[2][k]);
                t32[(3 + k) * (size_t)n + i] = (float)(p[1][k] - p[2][k]);
                t32[(6 + k) * (size_t)n + i] = (float)nr[k];
            }
            t32[9 * (size_t)n + i] = (float)(2.0 * ar);
        } else {
            for (int a = 0; a < 4; ++a)
                for (int k = 0; k < 3; ++k) q32[(3 * a + k) * (size_t)n + i] = (float)(p[a][k] - c[k]);
        }
    }
    bem_mesh_s *m = new bem_mesh_s();
    cudaGetDevice(&m->device);
    m->n = n;
    m->nvert = nvert;
    m->ext_of_int = order;
    m->int_of_ext = int_of_ext;
    auto up = [&](auto **dst, const auto &src) -> cudaError_t {
        cudaError_t e = dalloc(dst, src.size());
        if (e != cudaSuccess) return e;
        return cudaMemcpy(*dst, src.data(), src.size() * sizeof(src[0]), cudaMemcpyHostToDevice);
    };
    cudaError_t e = up(&m->d_nvert, nvert);
    if (e == cudaSuccess) e = up(&m->d_v64, v64);
    if (e == cudaSuccess) e = up(&m->d_c64, c64);
    if (e == cudaSuccess) e = up(&m->d_n64, n64);
    if (e == cudaSuccess) e = up(&m->d_area, area);
    if (e == cudaSuccess) e = up(&m->d_sqa, sqa);
    if (e == cudaSuccess) e = up(&m->d_chi, chi);
    if (e == cudaSuccess) e = up(&m->d_clo, clo);
    if (e == cudaSuccess) e = up(&m->d_t32, t32);
    if (e == cudaSuccess) e = up(&m->d_q32, q32);
    if (e == cudaSuccess) e = up(&m->d_isqa, isqa);
    if (e == cudaSuccess) e = up(&m->d_n32, n32);
    if (e == cudaSuccess) {
        std::vector<float4> row4(3 * (size_t)n);
        for (int i = 0; i < n; ++i) {
            row4[3 * (size_t)i] = make_float4(chi[i], chi[(size_t)n + i], chi[2 * (size_t)n + i], 0.f);
            row4[3 * (size_t)i + 1] = make_float4(clo[i], clo[(size_t)n + i], clo[2 * (size_t)n + i], 0.f);
            row4[3 * (size_t)i + 2] = make_float4(n32[i], n32[(size_t)n + i], n32[2 * (size_t)n + i], 0.f);
        }
        e = up(&m->d_row4, row4);
    }
    // symmetry images: one allocation, laid out as DevSym describes
    if (e == cudaSuccess && sym.nref > 1) {
        const size_t ni = (size_t)(sym.nref - 1) * (size_t)n;
        e = bem::dev_malloc(&m->d_img, bem::image_table_bytes(n, sym.nref));
        if (e == cudaSuccess) {
            bem::ImageTables it;
            it.v64 = (double *)m->d_img;
            it.c64 = it.v64 + 12 * ni;
            it.chi = (float *)(it.c64 + 3 * ni);
            it.clo = it.chi + 3 * ni;
            it.t32 = it.clo + 3 * ni;
            it.q32 = it.t32 + 10 * ni;
            sym.v64 = it.v64; sym.c64 = it.c64; sym.chi = it.chi; sym.clo = it.clo;
            sym.t32 = it.t32; sym.q32 = it.q32;
            m->sym = sym;
            e = bem::launch_image_tables(m->view(), it, 0);
        }
    } else {
        m->sym = sym;
    }
    // near list (geometry only, reused by every frequency): one pass into a
    // list sized for 48 pairs per element and image, a second with the exact
    // size only if that was too small
    unsigned long long *d_cnt = nullptr, cnt = 0;
    unsigned long long cap = 48ull * (unsigned long long)n * (unsigned long long)sym.nref;
    void *d_nls = nullptr;   // bounding spheres of the near-list column blocks
    if (e == cudaSuccess) e = bem::dev_malloc(&d_nls, bem::near_list_scratch_bytes(n, sym.nref));
    if (e == cudaSuccess) e = dalloc(&d_cnt, 1);
    for (int pass = 0; pass < 2 && e == cudaSuccess; ++pass) {
        if (e == cudaSuccess) e = dalloc(&m->d_near, (size_t)cap);
        if (e == cudaSuccess) e = cudaMemset(d_cnt, 0, sizeof(unsigned long long));
        if (e == cudaSuccess) e = bem::launch_near_list(m->view(), d_nls, m->d_near, cap, d_cnt, 0);
        if (e == cudaSuccess) e = cudaMemcpy(&cnt, d_cnt, sizeof(cnt), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess || cnt <= cap) break;
        bem::dev_free(m->d_near);
        m->d_near = nullptr;
        cap = cnt;
    }
    bem::dev_free(d_cnt);
    bem::dev_free(d_nls);
    if (e == cudaSuccess && cnt > cap) {
        delete m;
        return fail(BEM_ERR_CUDA, "near list: %llu pairs, list of %llu", cnt, cap);
    }
    m->n_near = (long long)cnt;
    if (e != cudaSuccess) {
        delete m;
        return fail(e == cudaErrorMemoryAllocation ? BEM_ERR_OUT_OF_HBM : BEM_ERR_CUDA, "mesh upload: %s",
                    cudaGetErrorString(e));
    }
    *out = m;
    return BEM_OK;
}

bem_status bem_mesh_destroy(bem_mesh_t mesh) {
    delete mesh;
    return BEM_OK;
}

bem_status bem_solver_create(bem_mesh_t mesh, const bem_solver_params *p, bem_solver_t *out) {
    if (!mesh || !out) return fail(BEM_ERR_INVALID, "null argument");
    *out = nullptr;
    bem_solver_params prm{};
    if (p) prm = *p;
    if (prm.precision != BEM_PREC_FP64 && prm.precision != BEM_PREC_MIXED)
        return fail(BEM_ERR_INVALID, "unknown precision %d", prm.precision);
    const int m = prm.restart > 0 ? prm.restart : 60;
    if (m > bem::kMaxRestart) return fail(BEM_ERR_INVALID, "restart length %d above the limit %d", m, bem::kMaxRestart);
    const int n = mesh->n;
    if (prm.no_precond < 0 || prm.no_precond > 3)
        return fail(BEM_ERR_INVALID, "no_precond %d is not 0, 1, 2 or 3", prm.no_precond);
    const bool pc = prm.no_precond != 1;
    const int prec = prm.precision == BEM_PREC_FP64 ? 0 : 1;
    const int n_rhs = prm.n_rhs > 0 ? prm.n_rhs : 1;
    if (n_rhs > bem::kMaxRhs) return fail(BEM_ERR_INVALID, "n_rhs %d above the limit %d", n_rhs, bem::kMaxRhs);
    if (prm.complex64_krylov < 0 || prm.complex64_krylov > 2)
        return fail(BEM_ERR_INVALID, "complex64_krylov %d is not 0, 1 or 2", prm.complex64_krylov);
    const int kcopy = prm.complex64_krylov;
    const size_t need = bem::solver_layout(n, prec, m, pc, nullptr, nullptr, n_rhs, nullptr, kcopy);
    size_t free_b = 0, total_b = 0;
    CU(cudaMemGetInfo(&free_b, &total_b));
    int dev = 0;
    CU(cudaGetDevice(&dev));
    free_b += bem::dev_cached_bytes(dev);   // cached blocks are free for this purpose
    double budget = prm.hbm_budget_bytes > 0 ? prm.hbm_budget_bytes : (double)free_b - 1.0e9;
    if ((double)need > budget)
        return fail(BEM_ERR_OUT_OF_HBM, "solver for %d unknowns needs %.3f GB, budget %.3f GB", n, need / 1e9,
                    budget / 1e9);
    std::unique_ptr<bem_solver_s> s(new bem_solver_s());
    s->mesh = mesh;
    s->n = n;
    s->prec = prm.precision;
    s->restart = m;
    s->max_iter = prm.max_iter > 0 ? prm.max_iter : 1000;
    s->tol = prm.tol > 0 ? prm.tol : 1e-9;
    s->lda = round_up((size_t)n, 32);
    s->precond = pc;
    s->pc_window = prm.no_precond == 0;
    s->pc_scaling = prm.no_precond == 3;
    cudaError_t e = cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking);
    for (auto &ev : s->ev)
        if (e == cudaSuccess) e = cudaEventCreate(&ev);
    if (e == cudaSuccess) e = bem::dev_malloc((void **)&s->block, need);
    if (e == cudaSuccess) {
        s->block_bytes = need;
        s->n_rhs = n_rhs;
        s->xr.resize(n_rhs - 1);
        s->xfreq.resize(n_rhs - 1);
        bem::solver_layout(n, prec, m, pc, s->block, &s->d, n_rhs, s->xr.data(), kcopy);
        e = cudaMemset(s->d.ctr, 0, 4 * sizeof(unsigned));
    }
    if (e != cudaSuccess)
        return fail(e == cudaErrorMemoryAllocation ? BEM_ERR_OUT_OF_HBM : BEM_ERR_CUDA, "solver allocation: %s",
                    cudaGetErrorString(e));
    *out = s.release();
    return BEM_OK;
}

bem_status bem_krylov_copy_info(bem_solver_t s, int32_t *blocks_per_row, int32_t *dense_blocks, double *mean_rank,
                                double *bytes_per_product) {
    if (!s) return fail(BEM_ERR_INVALID, "null argument");
    const int nb = s->d.blr_nb;
    if (nb <= 0) return fail(BEM_ERR_INVALID, "the solver has no block low-rank Krylov copy");
    std::vector<int> rk((size_t)nb * nb);
    CU(cudaStreamSynchronize(s->st));
    CU(cudaMemcpy(rk.data(), s->d.blr_rank, rk.size() * sizeof(int), cudaMemcpyDeviceToHost));
    const int n = s->n, nchunk = bem::mv_chunks(n);
    long long dense = 0, lr = 0, rsum = 0;
    double bytes = 0.0;
    std::vector<char> item_dense((size_t)nb * nchunk, 0);
    for (int I = 0; I < nb; ++I)
        for (int J = 0; J < nb; ++J) {
            const int r = rk[(size_t)I * nb + J];
            const double m = std::min(bem::kBlrB, n - I * bem::kBlrB), c = std::min(bem::kBlrB, n - J * bem::kBlrB);
            if (r < 0) {
                ++dense;
                bytes += m * c * 4.0;   // fp16 pairs of the fp16 copy
                item_dense[(size_t)I * nchunk + J * bem::kBlrB / bem::kMvChunk] = 1;
            } else {
                ++lr;
                rsum += r;
                bytes += (double)r * (2.0 * bem::kBlrB * 4.0 + 4.0);   // fp16 U_l, V_l and the scale
            }
        }
    // per item (block row x column chunk): its chunk of the input and, with a
    // dense block, the rows' scales; per row and chunk: one float partial
    for (int I = 0; I < nb; ++I)
        for (int c = 0; c < nchunk; ++c)
            bytes += bem::kMvChunk * 8.0 + (item_dense[(size_t)I * nchunk + c] ? bem::kBlrB * 4.0 : 0.0);
    bytes += (double)n * nchunk * 8.0;
    if (blocks_per_row) *blocks_per_row = nb;
    if (dense_blocks) *dense_blocks = (int32_t)dense;
    if (mean_rank) *mean_rank = lr > 0 ? (double)rsum / (double)lr : 0.0;
    if (bytes_per_product) *bytes_per_product = bytes;
    return BEM_OK;
}

bem_status bem_solver_destroy(bem_solver_t s) {
    delete s;
    return BEM_OK;
}

bem_status bem_solver_set_params(bem_solver_t s, const bem_solver_params *p) {
    if (!s || !p) return fail(BEM_ERR_INVALID, "null argument");
    if (p->max_iter > 0) s->max_iter = p->max_iter;
    if (p->tol > 0) s->tol = p->tol;
    return BEM_OK;
}

bem_status bem_assemble(bem_solver_t s, const bem_frequency_desc *f) {
    if (!s || !f) return fail(BEM_ERR_INVALID, "null argument");
    bem_status rc = upload_freq(s, f, s->st);
    if (rc != BEM_OK) return rc;
    bem_status one = BEM_OK;
    return assemble_group(&s, 1, s->st, s->d.ctr, s->ev[0], s->ev[1], &one);
}

// Restarted GMRES (bem_gmres.cu).  Each cycle starts from the explicitly
// computed residual r = b - A x, so with BEM_PREC_MIXED every cycle is one
// step of iterative refinement: the inner Arnoldi process (FP64 vectors,
// classical Gram-Schmidt with one re-orthogonalisation, FP64 inner products)
// uses the FP32 product with the fp16 copy of A (or with the complex64 matrix)
// and stops once it has gained three (five) digits; the outer residual is
// evaluated from the complex64 matrix, with error-free products in the first
// cycle and as r -= A d afterwards.
bem_status bem_solve(bem_solver_t s, bem_solve_info *info) {
    if (!s) return fail(BEM_ERR_INVALID, "null solver");
    if (!s->have_freq) return fail(BEM_ERR_INVALID, "bem_solve before bem_assemble");
    if (s->factored) return fail(BEM_ERR_INVALID, "bem_solve: the matrix was factored by bem_solve_direct; assemble again");
    bem_status one = BEM_OK;
    bem_status rc = solve_group(&s, 1, solver_engine(s), s->st, s->ev[2], s->ev[3], &one);
    if (info) *info = s->info;
    return rc;
}

bem_status bem_get_solution(bem_solver_t s, double *x_host) {
    if (!s || !x_host) return fail(BEM_ERR_INVALID, "null argument");
    return solution_to_host(s, s->st, x_host);
}

bem_status bem_get_system(bem_solver_t s, int32_t row0, int32_t row1, double *a_host, double *b_host) {
    if (!s) return fail(BEM_ERR_INVALID, "null solver");
    if (row0 < 0 || row1 > s->n || row0 > row1) return fail(BEM_ERR_INVALID, "bad row range");
    const int n = s->n;
    const std::vector<int> &ie = s->mesh->int_of_ext, &ext = s->mesh->ext_of_int;
    if (a_host && row1 > row0) {
        // rows and columns in the caller's element order
        const size_t esz = s->prec == BEM_PREC_FP64 ? 16 : 8;
        std::vector<unsigned char> row(esz * (size_t)n);
        for (int r = row0; r < row1; ++r) {
            const int ir = ie[r];
            CU(cudaMemcpyAsync(row.data(), (const char *)s->d.A + (size_t)ir * s->lda * esz, esz * n,
                               cudaMemcpyDeviceToHost, s->st));
            CU(cudaStreamSynchronize(s->st));
            double *out = a_host + 2 * (size_t)(r - row0) * n;
            for (int ic = 0; ic < n; ++ic) {
                double re, im;
                if (esz == 16) {
                    re = ((const double *)row.data())[2 * (size_t)ic];
                    im = ((const double *)row.data())[2 * (size_t)ic + 1];
                } else {
                    re = ((const float *)row.data())[2 * (size_t)ic];
                    im = ((const float *)row.data())[2 * (size_t)ic + 1];
                }
                out[2 * (size_t)ext[ic]] = re;
                out[2 * (size_t)ext[ic] + 1] = im;
            }
        }
    }
    if (b_host) {
        std::vector<double> t(2 * (size_t)n);
        bem_status rc = fetch(s->st, s->d.b, t.data(), t.size() * sizeof(double));
        if (rc != BEM_OK) return rc;
        for (int i = 0; i < n; ++i) {
            b_host[2 * (size_t)ext[i]] = t[2 * (size_t)i];
            b_host[2 * (size_t)ext[i] + 1] = t[2 * (size_t)i + 1];
        }
    }
    return BEM_OK;
}

bem_status bem_project(bem_solver_t s, int32_t n_pts, const double *pts, double *pot_out, double *grad_out) {
    if (!s) return fail(BEM_ERR_INVALID, "null solver");
    if (!s->solved) return fail(BEM_ERR_INVALID, "bem_project before bem_solve");
    if (n_pts < 0 || (n_pts > 0 && (!pts || !pot_out))) return fail(BEM_ERR_INVALID, "bad point arrays");
    bem_status one = BEM_OK;
    return project_group(&s, 1, &n_pts, &pts, &pot_out, &grad_out, s->st, s->ev[4], s->ev[5], &one);
}

bem_status bem_solve_frequency(bem_solver_t s, const bem_frequency_desc *f, int32_t n_pts, const double *pts,
                               double *x_out, double *pot_out, double *grad_out, bem_solve_info *info) {
    bem_status rc = bem_assemble(s, f);
    if (rc != BEM_OK) return rc;
    rc = bem_solve(s, info);
    if (rc != BEM_OK && rc != BEM_ERR_NOT_CONVERGED) return rc;
    bem_status solve_rc = rc;
    if (x_out) {
        rc = bem_get_solution(s, x_out);
        if (rc != BEM_OK) return rc;
    }
    rc = bem_project(s, n_pts, pts, pot_out, grad_out);
    if (rc != BEM_OK) return rc;
    if (info) *info = s->info;
    return solve_rc;
}

bem_status bem_solve_multi(bem_solver_t s, int32_t R, const bem_frequency_desc *freqs, int32_t n_pts,
                           const double *pts, double *const *x_out, double *const *pot_out, double *const *grad_out,
                           bem_solve_info *infos) {
    if (!s || !freqs) return fail(BEM_ERR_INVALID, "null argument");
    if (R < 1 || R > s->n_rhs)
        return fail(BEM_ERR_INVALID, "%d right-hand sides, the solver holds %d (bem_solver_params.n_rhs)", R, s->n_rhs);
    if (n_pts < 0 || (n_pts > 0 && !pts)) return fail(BEM_ERR_INVALID, "bad point arrays");
    cudaStream_t st = s->st;
    for (int r = 0; r < R; ++r) {
        bem_status rc = upload_freq(s, &freqs[r], st, r);
        if (rc != BEM_OK) return rc;
    }
    // the matrix once, the R right-hand sides in one launch
    CU(cudaMemsetAsync(s->d.status, 0, sizeof(int), st));
    CU(cudaEventRecord(s->ev[0], st));
    {
        std::unique_ptr<bem::AsmBatch> t(new bem::AsmBatch());
        t->B = 1;
        t->sys[0] = s->asys(0);
        bem::asm_batch_finish(*t);
        CU(bem::launch_assemble(*t, s->prec == BEM_PREC_FP64 ? 0 : 1, s->d.ctr, st));
        t->B = R;
        for (int r = 0; r < R; ++r) t->sys[r] = s->asys(r);
        bem::asm_batch_finish(*t);
        CU(bem::launch_rhs(*t, st));
    }
    CU(cudaEventRecord(s->ev[1], st));
    int code = 0;
    CU(cudaMemcpyAsync(&code, s->d.status, sizeof(int), cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    float ams = 0.f;
    CU(cudaEventElapsedTime(&ams, s->ev[0], s->ev[1]));
    s->info.assemble_ms = ams;
    s->info.n_near_pairs = (int64_t)(s->mesh->n_near - s->n);
    if (code != 0) return fail(BEM_ERR_SUBDIVISION, "%s", subdivision_message(code));
    s->have_freq = true;
    s->factored = false;
    s->solved = false;
    // preconditioner of the shared matrix, x = 0, then the R systems in lockstep
    CU(cudaEventRecord(s->ev[2], st));
    bem_status rc = precond_group(&s, 1, st);
    if (rc != BEM_OK) return rc;
    std::vector<bem::KSys> sys(R);
    std::vector<bem::KState> init(R);
    for (int r = 0; r < R; ++r) {
        if (r > 0) CU(cudaMemsetAsync(s->buf(r).x, 0, sizeof(double2) * s->n, st));
        sys[r] = s->ksys(r);
        init[r] = s->kinit();
    }
    bem::Engine *eng = solver_engine(s);
    CU(eng->set_batch(sys, init));
    bool all_done = false;
    for (long long body = 0; body < 2LL * s->max_iter + 64 && !all_done; ++body) {
        const cudaError_t be = eng->run_body();
        if (be == cudaErrorLaunchTimeout)
            return fail(BEM_ERR_DEVICE_TIMEOUT, "matrix-vector product: a bounded device wait gave up");
        CU(be);
        all_done = true;
        for (int r = 0; r < R; ++r)
            if (eng->states()[r].phase != bem::kPhaseFinished) all_done = false;
    }
    CU(cudaEventRecord(s->ev[3], st));
    CU(cudaEventSynchronize(s->ev[3]));
    float sms = 0.f;
    CU(cudaEventElapsedTime(&sms, s->ev[2], s->ev[3]));
    s->info.solve_ms = sms;
    s->info.matvec_ms = eng->timing_ok() ? eng->matvec_ms() : 0.0;
    s->solved = true;
    bem_status first = BEM_OK;
    std::vector<bem::KState> fin(eng->states(), eng->states() + R);
    for (int r = 0; r < R; ++r) {
        bem_status q = fin[r].phase == bem::kPhaseFinished ? map_result(fin[r])
                                                           : fail(BEM_ERR_DEVICE_TIMEOUT, "GMRES did not finish");
        if (q != BEM_OK && first == BEM_OK) first = q;
    }
    // projection of all right-hand sides
    rc = ensure_points(s, n_pts);
    if (rc != BEM_OK) return rc;
    CU(cudaMemsetAsync(s->d.status, 0, sizeof(int), st));
    CU(cudaEventRecord(s->ev[4], st));
    if (n_pts > 0) CU(cudaMemcpyAsync(s->pts, pts, sizeof(double) * 3 * n_pts, cudaMemcpyHostToDevice, st));
    {
        std::unique_ptr<bem::ProjBatch> t(new bem::ProjBatch());
        t->B = R;
        for (int r = 0; r < R; ++r)
            t->sys[r] = s->prsys(n_pts, s->pts, s->pot + 2 * (size_t)n_pts * r, s->grad + 6 * (size_t)n_pts * r, r);
        bem::proj_batch_finish(*t);
        CU(bem::launch_fields(*t, st));
        // mixed precision: one kernel evaluation per (point, element) pair
        // for up to 8 right-hand sides at a time
        if (s->prec == BEM_PREC_MIXED && R >= 2) {
            std::unique_ptr<bem::ProjBatch> u(new bem::ProjBatch());
            for (int c0 = 0; c0 < R; c0 += 8) {
                u->B = std::min(8, R - c0);
                for (int r = 0; r < u->B; ++r) u->sys[r] = t->sys[c0 + r];
                bem::proj_batch_finish(*u);
                CU(bem::launch_project_multi(*u, st));
            }
        } else {
            CU(bem::launch_project(*t, s->prec == BEM_PREC_FP64 ? 0 : 1, st));
        }
    }
    CU(cudaEventRecord(s->ev[5], st));
    for (int r = 0; r < R && n_pts > 0; ++r) {
        if (pot_out && pot_out[r])
            CU(cudaMemcpyAsync(pot_out[r], s->pot + 2 * (size_t)n_pts * r, sizeof(double) * 2 * n_pts,
                               cudaMemcpyDeviceToHost, st));
        if (grad_out && grad_out[r])
            CU(cudaMemcpyAsync(grad_out[r], s->grad + 6 * (size_t)n_pts * r, sizeof(double) * 6 * n_pts,
                               cudaMemcpyDeviceToHost, st));
    }
    CU(cudaMemcpyAsync(&code, s->d.status, sizeof(int), cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    float pms = 0.f;
    CU(cudaEventElapsedTime(&pms, s->ev[4], s->ev[5]));
    s->info.project_ms = pms;
    if (code != 0) return fail(BEM_ERR_SUBDIVISION, "evaluation point too close to the boundary: subdivision limit");
    for (int r = 0; r < R; ++r) {
        if (x_out && x_out[r]) {
            rc = solution_to_host(s, st, x_out[r], r);
            if (rc != BEM_OK) return rc;
        }
        if (infos) {
            infos[r] = s->info;
            infos[r].iterations = fin[r].iters;
            infos[r].restarts = fin[r].cycles;
            infos[r].rel_residual = fin[r].rel;
            infos[r].n_matvec = fin[r].n_mv;
        }
    }
    if (first != BEM_OK) {
        for (int r = 0; r < R; ++r)
            if (fin[r].result != bem::kResConverged) return map_result(fin[r]);
    }
    return BEM_OK;
}

bem_status bem_solve_batch(int32_t count, const bem_solver_t *solvers, const bem_frequency_desc *freqs,
                           const int32_t *n_pts, const double *const *pts, double *const *x_out,
                           double *const *pot_out, double *const *grad_out, bem_solve_info *infos,
                           bem_status *statuses) {
    if (count < 0 || (count > 0 && (!solvers || !freqs))) return fail(BEM_ERR_INVALID, "bad batch arrays");
    if (count == 0) return BEM_OK;
    for (int i = 0; i < count; ++i) {
        if (!solvers[i]) return fail(BEM_ERR_INVALID, "solver %d is null", i);
        for (int j = 0; j < i; ++j)
            if (solvers[j] == solvers[i]) return fail(BEM_ERR_INVALID, "solver %d appears twice in the batch", i);
        const int np = n_pts ? n_pts[i] : 0;
        if (np < 0 || (np > 0 && (!pts || !pts[i] || !pot_out || !pot_out[i])))
            return fail(BEM_ERR_INVALID, "bad point arrays of instance %d", i);
    }
    BatchCtx *ctx = nullptr;
    bem_status rc = batch_ctx(&ctx);
    if (rc != BEM_OK) return rc;
    for (int i = 0; i < count; ++i) CU(cudaStreamSynchronize(solvers[i]->st));
    std::vector<bem_status> rcs(count, BEM_OK), tmp(count, BEM_OK);
    bem_status first = BEM_OK;
    auto note = [&](int i, bem_status r) {
        if (r != BEM_OK && rcs[i] == BEM_OK) rcs[i] = r;
        if (r != BEM_OK && first == BEM_OK) first = r;
    };
    // per precision: one group for the assembly, the solve and the projection
    for (int prec = 0; prec < 2; ++prec) {
        std::vector<int> idx;
        for (int i = 0; i < count; ++i)
            if ((solvers[i]->prec == BEM_PREC_FP64 ? 0 : 1) == prec) idx.push_back(i);
        if (idx.empty()) continue;
        std::vector<bem_solver_t> g;
        for (int i : idx) {
            bem_status r = upload_freq(solvers[i], &freqs[i], ctx->st);
            if (r != BEM_OK) note(i, r);
            else g.push_back(solvers[i]);
        }
        if (g.empty()) continue;
        std::vector<int> gi;
        for (int i : idx)
            if (rcs[i] == BEM_OK) gi.push_back(i);
        const int cnt = (int)g.size();
        rc = assemble_group(g.data(), cnt, ctx->st, ctx->ctr, ctx->ev[0], ctx->ev[1], tmp.data());
        if (rc == BEM_ERR_CUDA) return rc;
        for (int q = 0; q < cnt; ++q) note(gi[q], tmp[q]);
        if (!ctx->eng[prec]) ctx->eng[prec].reset(new bem::Engine(prec, ctx->st));
        rc = solve_group(g.data(), cnt, ctx->eng[prec].get(), ctx->st, ctx->ev[2], ctx->ev[3], tmp.data());
        if (rc == BEM_ERR_CUDA || rc == BEM_ERR_DEVICE_TIMEOUT) return rc;
        for (int q = 0; q < cnt; ++q) note(gi[q], tmp[q]);
        std::vector<int32_t> np(cnt, 0);
        std::vector<const double *> pp(cnt, nullptr);
        std::vector<double *> po(cnt, nullptr), pg(cnt, nullptr);
        for (int q = 0; q < cnt; ++q) {
            const int i = gi[q];
            np[q] = n_pts ? n_pts[i] : 0;
            pp[q] = np[q] ? pts[i] : nullptr;
            po[q] = pot_out ? pot_out[i] : nullptr;
            pg[q] = grad_out ? grad_out[i] : nullptr;
        }
        rc = project_group(g.data(), cnt, np.data(), pp.data(), po.data(), pg.data(), ctx->st, ctx->ev[4],
                           ctx->ev[5], tmp.data());
        if (rc == BEM_ERR_CUDA) return rc;
        for (int q = 0; q < cnt; ++q) note(gi[q], tmp[q]);
        for (int q = 0; q < cnt; ++q) {
            const int i = gi[q];
            if (x_out && x_out[i]) {
                bem_status r = solution_to_host(g[q], ctx->st, x_out[i]);
                if (r != BEM_OK) return r;
            }
        }
    }
    for (int i = 0; i < count; ++i) {
        if (infos) infos[i] = solvers[i]->info;
        if (statuses) statuses[i] = rcs[i];
    }
    if (first != BEM_OK) {
        // keep the message of the first failing instance
        for (int i = 0; i < count; ++i)
            if (rcs[i] != BEM_OK) return rcs[i];
    }
    return BEM_OK;
}

}  // extern "C"

namespace bem {

// Inputs of the projection kernels held by a solved solver (for
// bem_project_static in bem_static.cu).
bool solver_projection_inputs(bem_solver_t s, int max_elem, ProjSys *out, int *prec, int *device) {
    if (!s) { g_err = "null solver"; return false; }
    *device = s->mesh->device;
    if (s->n > max_elem) {
        char buf[160];
        snprintf(buf, sizeof(buf), "bem_project_static: %d boundary elements, limit BEM_STATIC_MAX_ELEMENTS = %d",
                 s->n, max_elem);
        g_err = buf;
        return false;
    }
    if (!s->solved) { g_err = "bem_project_static before bem_solve"; return false; }
    *out = s->prsys(0, nullptr, nullptr, nullptr);
    *prec = s->prec;
    return true;
}

void set_error(const char *msg) { g_err = msg; }

}  // namespace bem
