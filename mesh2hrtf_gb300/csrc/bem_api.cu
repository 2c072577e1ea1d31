// bem_api.cu - the C ABI of include/bem_gb300.h: handles, device memory,
// HBM admission, the restarted GMRES driver and the per-frequency sequence.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/bem_gb300.h"
#include "bem_internal.h"

using cd = std::complex<double>;

namespace {

thread_local std::string g_err;

bem_status fail(bem_status st, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    return st;
}

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
    return cudaMalloc((void **)p, count * sizeof(T));
}

size_t round_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

}  // namespace

// ------------------------------------------------------------------ mesh
struct bem_mesh_s {
    int device = 0;
    int n = 0;
    std::vector<int> nvert;         // internal order
    std::vector<int> ext_of_int;    // internal unknown -> caller's element index
    std::vector<int> int_of_ext;
    // device buffers
    int *d_nvert = nullptr;
    double *d_v64 = nullptr, *d_c64 = nullptr, *d_n64 = nullptr, *d_area = nullptr, *d_sqa = nullptr;
    float *d_chi = nullptr, *d_clo = nullptr, *d_t32 = nullptr, *d_q32 = nullptr, *d_isqa = nullptr;
    float *d_n32 = nullptr;
    int2 *d_near = nullptr;         // pairs integrated with subdivision + self pairs
    long long n_near = 0;
    bem::DevMeshView view() const {
        bem::DevMeshView v;
        v.n = n; v.nvert = d_nvert; v.v64 = d_v64; v.c64 = d_c64; v.n64 = d_n64; v.area64 = d_area;
        v.sqa64 = d_sqa; v.chi = d_chi; v.clo = d_clo; v.t32 = d_t32; v.q32 = d_q32; v.isqa32 = d_isqa;
        v.n32 = d_n32;
        return v;
    }
    ~bem_mesh_s() {
        cudaFree(d_nvert); cudaFree(d_v64); cudaFree(d_c64); cudaFree(d_n64); cudaFree(d_area);
        cudaFree(d_sqa); cudaFree(d_chi); cudaFree(d_clo); cudaFree(d_t32); cudaFree(d_q32); cudaFree(d_isqa);
        cudaFree(d_near); cudaFree(d_n32);
    }
};

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

// ---------------------------------------------------------------- solver
struct bem_solver_s {
    bem_mesh_t mesh = nullptr;
    int n = 0;
    int prec = 0;
    int restart = 60;
    int max_iter = 1000;
    double tol = 1e-9;
    size_t lda = 0;
    cudaStream_t st = nullptr;
    cudaEvent_t ev[8] = {};
    void *A = nullptr;
    double *b = nullptr, *x = nullptr, *r = nullptr, *w = nullptr, *V = nullptr;
    double *hd = nullptr, *hsum = nullptr, *nrm = nullptr, *ydev = nullptr;
    double *Hd = nullptr, *csd = nullptr, *snd = nullptr, *gd = nullptr, *partial = nullptr;
    bem::GmresCtrl *ctrl = nullptr;
    std::vector<cudaEvent_t> mv_ev;   // per Arnoldi step: before/after the matvec
    void *xf = nullptr;
    void *Minv = nullptr, *Mwork = nullptr;
    bool precond = true, have_precond = false;
    double *z = nullptr;
    int *status = nullptr;
    unsigned long long *n_near = nullptr;
    // per-frequency device data
    int *f_bct = nullptr, *f_cols = nullptr;
    double *f_bcv = nullptr, *f_adm = nullptr, *f_src = nullptr;
    bem::DevFreq freq{};
    bool have_freq = false;
    bool solved = false;
    // fields and projection
    double *phi = nullptr, *vel = nullptr;
    int *ivi = nullptr;
    double *pts = nullptr, *pot = nullptr, *grad = nullptr;
    int pts_cap = 0;
    // pinned staging
    double *h_pin = nullptr;
    bem_solve_info info{};
    ~bem_solver_s() {
        if (st) cudaStreamSynchronize(st);
        cudaFree(A); cudaFree(b); cudaFree(x); cudaFree(r); cudaFree(w); cudaFree(V); cudaFree(hd);
        cudaFree(hsum); cudaFree(nrm); cudaFree(ydev); cudaFree(xf); cudaFree(status); cudaFree(n_near);
        cudaFree(Minv); cudaFree(Mwork); cudaFree(z);
        cudaFree(Hd); cudaFree(csd); cudaFree(snd); cudaFree(gd); cudaFree(partial); cudaFree(ctrl);
        for (auto &e : mv_ev)
            if (e) cudaEventDestroy(e);
        cudaFree(f_bct); cudaFree(f_cols); cudaFree(f_bcv); cudaFree(f_adm); cudaFree(f_src);
        cudaFree(phi); cudaFree(vel); cudaFree(ivi); cudaFree(pts); cudaFree(pot); cudaFree(grad);
        if (h_pin) cudaFreeHost(h_pin);
        for (auto &e : ev)
            if (e) cudaEventDestroy(e);
        if (st) cudaStreamDestroy(st);
    }
};

extern "C" {

const char *bem_last_error(void) { return g_err.c_str(); }

const char *bem_version(void) { return "mesh2hrtf_gb300 1.0 (sm_103a)"; }

int64_t bem_kernel_launches(void) { return (int64_t)bem::launches(); }

bem_status bem_set_device(int32_t device) {
    CU(cudaSetDevice(device));
    return ensure_device_init();
}

double bem_footprint_bytes(int32_t n_elem, int32_t precision, int32_t restart) {
    const double n = (double)n_elem;
    const double lda = (double)round_up((size_t)std::max(n_elem, 1), 32);
    const double esz = precision == BEM_PREC_FP64 ? 16.0 : 8.0;
    const int m = restart > 0 ? restart : 60;
    // matrix + Krylov basis + 5 work vectors + split x + fields (phi, 4 vel)
    // + block-Jacobi inverses
    return n * lda * esz + (m + 1) * n * 16.0 + 5 * n * 16.0 + n * 16.0 + 5 * n * 16.0 + n * 64.0 +
           (double)bem::precond_bytes(n_elem, precision);
}

bem_status bem_mesh_create(const bem_mesh_desc *d, bem_mesh_t *out) {
    if (!d || !out) return fail(BEM_ERR_INVALID, "null argument");
    *out = nullptr;
    if (d->n_elem <= 0 || d->n_nodes <= 0 || !d->nodes || !d->conn || !d->nvert)
        return fail(BEM_ERR_INVALID, "mesh needs elements, nodes, connectivity and vertex counts");
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
    // near list: count, allocate, fill (geometry only, reused by every frequency)
    unsigned long long *d_cnt = nullptr, cnt = 0;
    if (e == cudaSuccess) e = dalloc(&d_cnt, 1);
    if (e == cudaSuccess) e = cudaMemset(d_cnt, 0, sizeof(unsigned long long));
    if (e == cudaSuccess) e = bem::launch_near_list(m->view(), nullptr, d_cnt, 0);
    if (e == cudaSuccess) e = cudaMemcpy(&cnt, d_cnt, sizeof(cnt), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = dalloc(&m->d_near, (size_t)cnt);
    if (e == cudaSuccess) e = cudaMemset(d_cnt, 0, sizeof(unsigned long long));
    if (e == cudaSuccess) e = bem::launch_near_list(m->view(), m->d_near, d_cnt, 0);
    unsigned long long cnt2 = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&cnt2, d_cnt, sizeof(cnt2), cudaMemcpyDeviceToHost);
    cudaFree(d_cnt);
    if (e == cudaSuccess && cnt2 != cnt) {
        delete m;
        return fail(BEM_ERR_CUDA, "near list: inconsistent counts %llu / %llu", cnt, cnt2);
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
    const int n = mesh->n;
    const int m = prm.restart > 0 ? prm.restart : 60;
    const double need = bem_footprint_bytes(n, prm.precision, m);
    size_t free_b = 0, total_b = 0;
    CU(cudaMemGetInfo(&free_b, &total_b));
    double budget = prm.hbm_budget_bytes > 0 ? prm.hbm_budget_bytes : (double)free_b - 1.0e9;
    if (need > budget)
        return fail(BEM_ERR_OUT_OF_HBM, "solver for %d unknowns needs %.3f GB, budget %.3f GB", n, need / 1e9,
                    budget / 1e9);
    bem_solver_s *s = new bem_solver_s();
    s->mesh = mesh;
    s->n = n;
    s->prec = prm.precision;
    s->restart = m;
    s->max_iter = prm.max_iter > 0 ? prm.max_iter : 1000;
    s->tol = prm.tol > 0 ? prm.tol : 1e-9;
    s->lda = round_up((size_t)n, 32);
    const size_t esz = s->prec == BEM_PREC_FP64 ? 16 : 8;
    auto cleanup = [&](cudaError_t e) {
        delete s;
        return fail(e == cudaErrorMemoryAllocation ? BEM_ERR_OUT_OF_HBM : BEM_ERR_CUDA, "solver allocation: %s",
                    cudaGetErrorString(e));
    };
    cudaError_t e = cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking);
    for (auto &ev : s->ev)
        if (e == cudaSuccess) e = cudaEventCreate(&ev);
    if (e == cudaSuccess) e = cudaMalloc(&s->A, (size_t)n * s->lda * esz);
    if (e == cudaSuccess) e = dalloc(&s->b, 2 * (size_t)n);
    if (e == cudaSuccess) e = dalloc(&s->x, 2 * (size_t)n);
    if (e == cudaSuccess) e = dalloc(&s->r, 2 * (size_t)n);
    if (e == cudaSuccess) e = dalloc(&s->w, 2 * (size_t)n);
    if (e == cudaSuccess) e = dalloc(&s->V, 2 * (size_t)n * (m + 1));
    if (e == cudaSuccess) e = dalloc(&s->hd, 2 * (size_t)(m + 2));
    if (e == cudaSuccess) e = dalloc(&s->hsum, 2 * (size_t)(m + 2));
    if (e == cudaSuccess) e = dalloc(&s->nrm, 4);
    if (e == cudaSuccess) e = dalloc(&s->ydev, 2 * (size_t)(m + 2));
    if (e == cudaSuccess) e = cudaMalloc(&s->xf, 16 * (size_t)n);
    s->precond = prm.no_precond == 0;
    if (s->precond) {
        const size_t pb = bem::precond_bytes(n, s->prec);
        const size_t half = s->prec == BEM_PREC_FP64 ? pb / 2 : pb;
        if (e == cudaSuccess) e = cudaMalloc(&s->Minv, half);
        if (e == cudaSuccess && s->prec == BEM_PREC_FP64) e = cudaMalloc(&s->Mwork, half);
        if (e == cudaSuccess) e = dalloc(&s->z, 2 * (size_t)n);
    }
    if (e == cudaSuccess) e = dalloc(&s->status, 1);
    if (e == cudaSuccess) e = dalloc(&s->n_near, 1);
    if (e == cudaSuccess) e = dalloc(&s->phi, 2 * (size_t)n);
    if (e == cudaSuccess) e = dalloc(&s->vel, 8 * (size_t)n);
    if (e == cudaSuccess) e = dalloc(&s->ivi, (size_t)n);
    if (e == cudaSuccess) e = dalloc(&s->Hd, 2 * (size_t)(m + 1) * m);
    if (e == cudaSuccess) e = dalloc(&s->csd, 2 * (size_t)m);
    if (e == cudaSuccess) e = dalloc(&s->snd, 2 * (size_t)m);
    if (e == cudaSuccess) e = dalloc(&s->gd, 2 * (size_t)(m + 1));
    if (e == cudaSuccess) e = dalloc(&s->partial, 2 * (size_t)(m + 2) * bem::dot_blocks(n));
    if (e == cudaSuccess) e = cudaMalloc(&s->ctrl, sizeof(bem::GmresCtrl));
    s->mv_ev.assign(2 * (size_t)m, nullptr);
    for (auto &ev : s->mv_ev)
        if (e == cudaSuccess) e = cudaEventCreate(&ev);
    if (e == cudaSuccess)
        e = cudaMallocHost(&s->h_pin, sizeof(double) * (2 * (size_t)(m + 1) * m + 2 * (size_t)(m + 4) + 8));
    if (e != cudaSuccess) return cleanup(e);
    *out = s;
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

static bem_status upload_freq(bem_solver_t s, const bem_frequency_desc *f) {
    const int n = s->n;
    if (!(f->wave_number > 0.0)) return fail(BEM_ERR_INVALID, "wave number must be > 0");
    if (f->n_point < 0 || f->n_plane < 0) return fail(BEM_ERR_INVALID, "negative source count");
    if ((f->n_point && (!f->point_xyz || !f->point_amp)) || (f->n_plane && (!f->plane_dir || !f->plane_amp)))
        return fail(BEM_ERR_INVALID, "source arrays missing");
    bem::DevFreq &F = s->freq;
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
    cudaFree(s->f_bct); cudaFree(s->f_cols); cudaFree(s->f_bcv); cudaFree(s->f_adm); cudaFree(s->f_src);
    s->f_bct = s->f_cols = nullptr;
    s->f_bcv = s->f_adm = s->f_src = nullptr;
    std::vector<int> cols;
    const std::vector<int> &ext = s->mesh->ext_of_int;
    std::vector<int> bct_int;
    if (f->bc_type) {
        for (int j = 0; j < n; ++j)
            if (f->bc_type[j] < 0 || f->bc_type[j] > 2)
                return fail(BEM_ERR_INVALID, "element %d: boundary condition type %d unsupported", j, f->bc_type[j]);
        bct_int.resize(n);
        for (int i = 0; i < n; ++i) bct_int[i] = f->bc_type[ext[i]];
        CU(dalloc(&s->f_bct, (size_t)n));
        CU(cudaMemcpyAsync(s->f_bct, bct_int.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s->st));
        CU(cudaStreamSynchronize(s->st));
        F.bc_type = s->f_bct;
    }
    if (f->bc_value) {
        std::vector<double> t(8 * (size_t)n);
        for (int i = 0; i < n; ++i) {
            const int j = ext[i];
            bool nz = false;
            for (int a = 0; a < 4; ++a) {
                const double re = f->bc_value[8 * (size_t)j + 2 * a], im = f->bc_value[8 * (size_t)j + 2 * a + 1];
                t[2 * ((size_t)a * n + i)] = re;
                t[2 * ((size_t)a * n + i) + 1] = im;
                // NumCalc's test: |value| > EPSY on the element's nodes (NC_EquationSystem.cpp:264-275)
                if (a < s->mesh->nvert[i] && std::sqrt(re * re + im * im) > 1.0e-14) nz = true;
            }
            if (nz) cols.push_back(i);
        }
        CU(dalloc(&s->f_bcv, t.size()));
        CU(cudaMemcpyAsync(s->f_bcv, t.data(), sizeof(double) * t.size(), cudaMemcpyHostToDevice, s->st));
        CU(cudaStreamSynchronize(s->st));
        F.bc_val = s->f_bcv;
    }
    if (f->admittance) {
        std::vector<double> t(2 * (size_t)n);
        for (int i = 0; i < n; ++i) {
            t[2 * (size_t)i] = f->admittance[2 * (size_t)ext[i]];
            t[2 * (size_t)i + 1] = f->admittance[2 * (size_t)ext[i] + 1];
        }
        CU(dalloc(&s->f_adm, 2 * (size_t)n));
        CU(cudaMemcpyAsync(s->f_adm, t.data(), sizeof(double) * 2 * n, cudaMemcpyHostToDevice, s->st));
        CU(cudaStreamSynchronize(s->st));
        F.adm = s->f_adm;
    }
    if (!cols.empty()) {
        CU(dalloc(&s->f_cols, cols.size()));
        CU(cudaMemcpyAsync(s->f_cols, cols.data(), sizeof(int) * cols.size(), cudaMemcpyHostToDevice, s->st));
        CU(cudaStreamSynchronize(s->st));
        F.bc_cols = s->f_cols;
        F.n_bc_cols = (int)cols.size();
    }
    const size_t nsrc = 5 * (size_t)f->n_point + 5 * (size_t)f->n_plane;
    if (nsrc) {
        // complex amplitudes first so that they start on 16-byte boundaries
        // (the kernels read them as double2), coordinates after them
        std::vector<double> src;
        src.reserve(nsrc);
        for (int i = 0; i < 2 * f->n_point; ++i) src.push_back(f->point_amp[i]);
        for (int i = 0; i < 2 * f->n_plane; ++i) src.push_back(f->plane_amp[i]);
        for (int i = 0; i < 3 * f->n_point; ++i) src.push_back(f->point_xyz[i]);
        for (int i = 0; i < 3 * f->n_plane; ++i) src.push_back(f->plane_dir[i]);
        CU(dalloc(&s->f_src, src.size()));
        CU(cudaMemcpyAsync(s->f_src, src.data(), sizeof(double) * src.size(), cudaMemcpyHostToDevice, s->st));
        CU(cudaStreamSynchronize(s->st));
        F.n_point = f->n_point;
        F.n_plane = f->n_plane;
        F.ps_amp = s->f_src;
        F.pw_amp = s->f_src + 2 * (size_t)f->n_point;
        F.ps_xyz = s->f_src + 2 * (size_t)f->n_point + 2 * (size_t)f->n_plane;
        F.pw_dir = F.ps_xyz + 3 * (size_t)f->n_point;
    }
    return BEM_OK;
}

bem_status bem_assemble(bem_solver_t s, const bem_frequency_desc *f) {
    if (!s || !f) return fail(BEM_ERR_INVALID, "null argument");
    bem_status rc = upload_freq(s, f);
    if (rc != BEM_OK) return rc;
    CU(cudaMemsetAsync(s->status, 0, sizeof(int), s->st));
    CU(cudaEventRecord(s->ev[0], s->st));
    CU(bem::launch_assemble(s->mesh->view(), s->freq, s->prec, s->A, s->lda, s->mesh->d_near, s->mesh->n_near,
                            s->status, s->st));
    CU(bem::launch_rhs(s->mesh->view(), s->freq, s->b, s->status, s->st));
    CU(cudaEventRecord(s->ev[1], s->st));
    int st_h = 0;
    CU(cudaMemcpyAsync(&st_h, s->status, sizeof(int), cudaMemcpyDeviceToHost, s->st));
    CU(cudaStreamSynchronize(s->st));
    const long long nn = s->mesh->n_near - s->n;   // subdivided pairs (self pairs excluded)
    float ms = 0.f;
    CU(cudaEventElapsedTime(&ms, s->ev[0], s->ev[1]));
    s->info.assemble_ms = ms;
    s->info.n_near_pairs = (int64_t)nn;
    s->have_freq = true;
    s->solved = false;
    if (st_h != 0)
        return fail(BEM_ERR_SUBDIVISION,
                    st_h == 1 ? "number of subelements which are subdivided in a loop must <= 15"
                              : "number of subelements must be < 220");
    return BEM_OK;
}

namespace {

// host copy of a device complex vector
bem_status fetch(bem_solver_t s, const double *dsrc, double *hdst, size_t ndoubles) {
    CU(cudaMemcpyAsync(hdst, dsrc, ndoubles * sizeof(double), cudaMemcpyDeviceToHost, s->st));
    CU(cudaStreamSynchronize(s->st));
    return BEM_OK;
}

}  // namespace

// Restarted GMRES.  Each cycle starts from the explicitly computed residual
// r = b - A x, so with BEM_PREC_MIXED every cycle is one step of iterative
// refinement: the inner Arnoldi process (FP64 vectors, CGS with one
// re-orthogonalisation, FP64 inner products) works with the fast FP32
// matrix-vector product and stops once it has gained five digits, and the
// outer residual is evaluated with the error-free-transformation product.
bem_status bem_solve(bem_solver_t s, bem_solve_info *info) {
    if (!s) return fail(BEM_ERR_INVALID, "null solver");
    if (!s->have_freq) return fail(BEM_ERR_INVALID, "bem_solve before bem_assemble");
    const int n = s->n, m = s->restart;
    const size_t ldv = 2 * (size_t)n;      // doubles between basis vectors
    const size_t ldc = (size_t)n;          // complex entries between basis vectors
    CU(cudaEventRecord(s->ev[2], s->st));
    // block-Jacobi inverses of this frequency's matrix
    s->have_precond = false;
    if (s->precond) {
        CU(cudaMemsetAsync(s->status, 0, sizeof(int), s->st));
        CU(bem::launch_block_inverse(s->prec, s->A, s->lda, n, s->Minv, s->Mwork, s->status, s->st));
        int sing = 0;
        CU(cudaMemcpyAsync(&sing, s->status, sizeof(int), cudaMemcpyDeviceToHost, s->st));
        CU(cudaStreamSynchronize(s->st));
        s->have_precond = sing == 0;   // a singular block: solve unpreconditioned
    }
    const bool pc = s->have_precond;
    CU(cudaMemsetAsync(s->x, 0, sizeof(double) * 2 * n, s->st));
    CU(bem::launch_norm2(s->b, n, s->nrm, s->st));
    double *hp = s->h_pin;
    bem_status rc = fetch(s, s->nrm, hp, 1);
    if (rc) return rc;
    const double bnorm = std::sqrt(hp[0]);
    int iters = 0, cycles = 0, n_mv = 0;
    double rel = 0.0, mv_ms = 0.0;
    bool converged = false;
    if (bnorm == 0.0 || !std::isfinite(bnorm)) {
        converged = bnorm == 0.0;
        if (!converged) return fail(BEM_ERR_INVALID, "right-hand side is not finite");
    } else {
        CU(cudaMemcpyAsync(s->r, s->b, sizeof(double) * 2 * n, cudaMemcpyDeviceToDevice, s->st));
        CU(cudaMemcpyAsync(s->nrm + 2, s->nrm, sizeof(double), cudaMemcpyDeviceToDevice, s->st));
        double beta = bnorm, prev_beta = 0.0;
        std::vector<cd> H((size_t)(m + 1) * m), g(m + 1), y(m);
        const int batch = 8;   // Arnoldi steps queued between convergence checks
        while (true) {
            ++cycles;
            // cycle set-up: V0 = r / beta, g = (beta, 0, ...), hsum = 0, ctrl
            CU(bem::launch_scale_inv(s->r, s->nrm + 2, s->V, n, s->st));
            CU(cudaMemsetAsync(s->gd, 0, sizeof(double) * 2 * (m + 1), s->st));
            CU(cudaMemsetAsync(s->hsum, 0, sizeof(double) * 2 * (m + 1), s->st));
            const double inner_floor = s->prec == BEM_PREC_MIXED ? 1e-5 * beta : 0.0;
            bem::GmresCtrl c0{0, 0, 0.0, std::max(s->tol * bnorm, inner_floor)};
            double *hc = hp + 2 * (size_t)(m + 1) * m + 2 * (size_t)(m + 4);
            std::memcpy(hc, &c0, sizeof(c0));
            hc[4] = beta;
            hc[5] = 0.0;
            CU(cudaMemcpyAsync(s->ctrl, hc, sizeof(c0), cudaMemcpyHostToDevice, s->st));
            CU(cudaMemcpyAsync(s->gd, hc + 4, sizeof(double) * 2, cudaMemcpyHostToDevice, s->st));
            const int *done = &s->ctrl->done;
            const int kmax = std::min(m, s->max_iter - iters);
            int k = 0, kdone = 0;
            bool cyc_done = false;
            while (k < kmax && !cyc_done) {
                const int k_end = std::min(kmax, k + batch);
                for (; k < k_end; ++k) {
                    double *vk = s->V + (size_t)k * ldv;
                    if (pc) {
                        CU(bem::launch_block_apply(s->prec, s->Minv, n, vk, s->z, s->st, done));
                        vk = s->z;
                    }
                    CU(cudaEventRecord(s->mv_ev[2 * k], s->st));
                    CU(bem::launch_matvec(s->prec, false, s->A, n, s->lda, vk, nullptr, s->w, s->xf, s->st, done));
                    CU(cudaEventRecord(s->mv_ev[2 * k + 1], s->st));
                    for (int pass = 0; pass < 2; ++pass) {   // classical Gram-Schmidt, twice
                        CU(bem::launch_multi_dot(s->V, ldc, k + 1, s->w, n, s->partial, s->hd, s->hsum, s->st, done));
                        CU(bem::launch_multi_axpy(s->V, ldc, k + 1, s->hd, s->w, n, s->st, done));
                    }
                    CU(bem::launch_multi_dot(s->w, ldc, 1, s->w, n, s->partial, s->nrm, nullptr, s->st, done));
                    CU(bem::launch_scale_inv(s->w, s->nrm, s->V + (size_t)(k + 1) * ldv, n, s->st, done));
                    CU(bem::launch_givens(k, m, s->hsum, s->nrm, s->Hd, s->csd, s->snd, s->gd, s->ctrl, s->st));
                }
                bem::GmresCtrl cs_h;
                CU(cudaMemcpyAsync(hc, s->ctrl, sizeof(cs_h), cudaMemcpyDeviceToHost, s->st));
                CU(cudaStreamSynchronize(s->st));
                std::memcpy(&cs_h, hc, sizeof(cs_h));
                kdone = cs_h.kdone;
                cyc_done = cs_h.done != 0;
                if (!std::isfinite(cs_h.res)) return fail(BEM_ERR_NOT_CONVERGED, "GMRES breakdown (non-finite residual)");
            }
            for (int q = 0; q < kdone; ++q) {
                float mv = 0.f;
                CU(cudaEventElapsedTime(&mv, s->mv_ev[2 * q], s->mv_ev[2 * q + 1]));
                mv_ms += mv;
                ++n_mv;
            }
            iters += kdone;
            const int kk = kdone;
            if (kk > 0) {
                // y = H^{-1} g on the host (kk x kk upper triangular)
                CU(cudaMemcpyAsync(hp, s->Hd, sizeof(double) * 2 * (size_t)(m + 1) * m, cudaMemcpyDeviceToHost, s->st));
                CU(cudaMemcpyAsync(hp + 2 * (size_t)(m + 1) * m, s->gd, sizeof(double) * 2 * (m + 1),
                                   cudaMemcpyDeviceToHost, s->st));
                CU(cudaStreamSynchronize(s->st));
                for (size_t q = 0; q < (size_t)(m + 1) * m; ++q) H[q] = cd(hp[2 * q], hp[2 * q + 1]);
                const double *gp = hp + 2 * (size_t)(m + 1) * m;
                for (int q = 0; q <= m; ++q) g[q] = cd(gp[2 * q], gp[2 * q + 1]);
                for (int i2 = kk - 1; i2 >= 0; --i2) {
                    cd acc = g[i2];
                    for (int l = i2 + 1; l < kk; ++l) acc -= H[(size_t)i2 * m + l] * y[l];
                    y[i2] = acc / H[(size_t)i2 * m + i2];
                }
                for (int l = 0; l < kk; ++l) { hp[2 * l] = y[l].real(); hp[2 * l + 1] = y[l].imag(); }
                CU(cudaMemcpyAsync(s->ydev, hp, sizeof(double) * 2 * kk, cudaMemcpyHostToDevice, s->st));
                if (pc) {
                    // x += M^{-1} (V y)
                    CU(cudaMemsetAsync(s->w, 0, sizeof(double) * 2 * n, s->st));
                    CU(bem::launch_update_x(s->V, (int)ldc, kk, s->ydev, s->w, n, s->st));
                    CU(bem::launch_block_apply(s->prec, s->Minv, n, s->w, s->z, s->st));
                    CU(bem::launch_axpy(s->z, s->x, n, s->st));
                } else {
                    CU(bem::launch_update_x(s->V, (int)ldc, kk, s->ydev, s->x, n, s->st));
                }
            }
            // explicit residual (the refinement step)
            CU(cudaEventRecord(s->ev[6], s->st));
            CU(bem::launch_matvec(s->prec, true, s->A, n, s->lda, s->x, s->b, s->r, s->xf, s->st));
            CU(cudaEventRecord(s->ev[7], s->st));
            CU(bem::launch_norm2(s->r, n, s->nrm + 2, s->st));
            rc = fetch(s, s->nrm + 2, hp, 1);
            if (rc) return rc;
            {
                float mv = 0.f;
                CU(cudaEventElapsedTime(&mv, s->ev[6], s->ev[7]));
                mv_ms += mv;
                ++n_mv;
            }
            prev_beta = beta;
            beta = std::sqrt(hp[0]);
            rel = beta / bnorm;
            if (!std::isfinite(rel)) return fail(BEM_ERR_NOT_CONVERGED, "GMRES breakdown (non-finite residual)");
            if (rel <= s->tol) { converged = true; break; }
            if (iters >= s->max_iter) break;
            if (cycles > 2 && beta > 0.9 * prev_beta && s->prec == BEM_PREC_MIXED) break;  // refinement stagnates
        }
    }
    CU(cudaEventRecord(s->ev[3], s->st));
    CU(cudaEventSynchronize(s->ev[3]));
    float ms = 0.f;
    CU(cudaEventElapsedTime(&ms, s->ev[2], s->ev[3]));
    s->info.solve_ms = ms;
    s->info.iterations = iters;
    s->info.restarts = cycles;
    s->info.rel_residual = rel;
    s->info.matvec_ms = mv_ms;
    s->info.n_matvec = n_mv;
    s->solved = true;
    if (info) *info = s->info;
    if (!converged)
        return fail(BEM_ERR_NOT_CONVERGED, "GMRES reached %d iterations, relative residual %.3e", iters, rel);
    return BEM_OK;
}

bem_status bem_get_solution(bem_solver_t s, double *x_host) {
    if (!s || !x_host) return fail(BEM_ERR_INVALID, "null argument");
    std::vector<double> t(2 * (size_t)s->n);
    bem_status rc = fetch(s, s->x, t.data(), t.size());
    if (rc != BEM_OK) return rc;
    const std::vector<int> &ext = s->mesh->ext_of_int;
    for (int i = 0; i < s->n; ++i) {
        x_host[2 * (size_t)ext[i]] = t[2 * (size_t)i];
        x_host[2 * (size_t)ext[i] + 1] = t[2 * (size_t)i + 1];
    }
    return BEM_OK;
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
            CU(cudaMemcpyAsync(row.data(), (const char *)s->A + (size_t)ir * s->lda * esz, esz * n,
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
        bem_status rc = fetch(s, s->b, t.data(), t.size());
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
    if (n_pts > s->pts_cap) {
        cudaFree(s->pts); cudaFree(s->pot); cudaFree(s->grad);
        s->pts = s->pot = s->grad = nullptr;
        s->pts_cap = 0;
        CU(dalloc(&s->pts, 3 * (size_t)n_pts));
        CU(dalloc(&s->pot, 2 * (size_t)n_pts));
        CU(dalloc(&s->grad, 6 * (size_t)n_pts));
        s->pts_cap = n_pts;
    }
    CU(cudaEventRecord(s->ev[4], s->st));
    CU(bem::launch_fields(s->mesh->view(), s->freq, s->x, s->phi, s->vel, s->ivi, s->st));
    if (n_pts > 0) {
        CU(cudaMemcpyAsync(s->pts, pts, sizeof(double) * 3 * n_pts, cudaMemcpyHostToDevice, s->st));
        CU(cudaMemsetAsync(s->status, 0, sizeof(int), s->st));
        CU(bem::launch_project(s->mesh->view(), s->freq, s->prec, s->phi, s->vel, s->ivi, n_pts, s->pts, s->pot,
                               s->grad, s->status, s->st));
        CU(cudaMemcpyAsync(pot_out, s->pot, sizeof(double) * 2 * n_pts, cudaMemcpyDeviceToHost, s->st));
        if (grad_out)
            CU(cudaMemcpyAsync(grad_out, s->grad, sizeof(double) * 6 * n_pts, cudaMemcpyDeviceToHost, s->st));
    }
    CU(cudaEventRecord(s->ev[5], s->st));
    int st_h = 0;
    CU(cudaMemcpyAsync(&st_h, s->status, sizeof(int), cudaMemcpyDeviceToHost, s->st));
    CU(cudaStreamSynchronize(s->st));
    float ms = 0.f;
    CU(cudaEventElapsedTime(&ms, s->ev[4], s->ev[5]));
    s->info.project_ms = ms;
    if (st_h != 0)
        return fail(BEM_ERR_SUBDIVISION, "evaluation point too close to the boundary: subdivision limit");
    return BEM_OK;
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

}  // extern "C"

namespace bem {

// Inputs of the projection kernels held by a solved solver (for
// bem_project_static in bem_static.cu).
bool solver_projection_inputs(bem_solver_t s, int max_elem, DevMeshView *m, DevFreq *f, int *prec,
                              const double **x, int *n) {
    if (!s) { g_err = "null solver"; return false; }
    if (s->n > max_elem) {
        char buf[160];
        snprintf(buf, sizeof(buf), "bem_project_static: %d boundary elements, limit BEM_STATIC_MAX_ELEMENTS = %d",
                 s->n, max_elem);
        g_err = buf;
        return false;
    }
    if (!s->solved) { g_err = "bem_project_static before bem_solve"; return false; }
    *m = s->mesh->view();
    *f = s->freq;
    *prec = s->prec;
    *x = s->x;
    *n = s->n;
    return true;
}

void set_error(const char *msg) { g_err = msg; }

}  // namespace bem
