// bem_kernels.cu - assembly, right-hand side and field-projection kernels.
//
// Assembly tile: a block of 8 warps covers 8 rows x 32 columns of A; each
// warp owns one row i (collocation point = centre of element i) and 32
// consecutive columns j (one per lane).  A lane classifies its pair with
// NumCalc's level-0 subdivision test; regular pairs are integrated in the
// lane with the Gauss order NumCalc would pick, pairs that NumCalc
// subdivides and the self pair are integrated afterwards by the whole warp,
// one after the other (warp_subdivide / warp_singular).  Each entry is
// written once, by its lane, as a coalesced row segment.
#include <type_traits>

#include "bem_internal.h"
#include "bem_pair.cuh"

namespace bem {

namespace {

template <typename T> struct Vec2;
template <> struct Vec2<double> { using type = double2; };
template <> struct Vec2<float> { using type = float2; };

__device__ __forceinline__ DevMesh to_dev(const DevMeshView &v) {
    DevMesh m;
    m.n = v.n; m.nvert = v.nvert; m.v64 = v.v64; m.c64 = v.c64; m.n64 = v.n64;
    m.area64 = v.area64; m.sqa64 = v.sqa64; m.chi = v.chi; m.clo = v.clo; m.t32 = v.t32;
    m.q32 = v.q32; m.isqa32 = v.isqa32; m.n32 = v.n32;
    return m;
}

__device__ __forceinline__ cplx<double> ld_c(const double *p, int idx) {
    double2 v = reinterpret_cast<const double2 *>(p)[idx];
    return {v.x, v.y};
}

// Approximate level-0 decision in float; returns false if the ratio lies too
// close to a threshold to decide without the exact FP64 value.
__device__ __forceinline__ bool classify_fast(float rf, bool &near, int &order) {
    const float tol = 2e-5f;
    if (fabsf(rf - 1.3f) <= tol * 1.3f) return false;
    near = rf < 1.3f;
    if (near) return true;
#pragma unroll
    for (int mm = 2; mm <= 5; ++mm) {
        const float t = c_quad.order_thrf[mm];
        if (fabsf(rf - t) <= tol * t) return false;
        if (rf >= t) { order = mm; return true; }
    }
    order = 6;
    return true;
}

// Regular pair in precision T with a fixed Gauss order (no subdivision):
// the single-subelement case of NC_RegularIntegration.
template <typename T> struct FarPair;

template <> struct FarPair<double> {
    static __device__ __forceinline__ KVals<double> run(const Elem64 &e, const double x[3], const double nx[3],
                                                        int order, double k, double wr) {
        KVals<double> acc;
        acc.G = acc.H = acc.HT = acc.E = cmk(0.0, 0.0);
        const int np = e.nv == 3 ? tri_count(order) : quad_count(order);
        for (int g = 0; g < np; ++g) {
            double s, t, w;
            if (e.nv == 3) {
                const int o = tri_offset(order) + g;
                s = c_quad.tri[o][0]; t = c_quad.tri[o][1]; w = c_quad.tri[o][2];
            } else {
                const int a = g / order, b = g - a * order;
                s = c_quad.glx[order][a]; t = c_quad.glx[order][b];
                w = c_quad.glw[order][a] * c_quad.glw[order][b];
            }
            QPoint<double> q;
            map_point(e, s, t, x, w, q);
            KVals<double> v = kernel_values(q, nx, k, wr);
            acc.G += v.G; acc.H += v.H; acc.HT += v.HT; acc.E += v.E;
        }
        return acc;
    }
};

template <> struct FarPair<float> {
    static __device__ __forceinline__ KVals<float> run(const Elem32 &e, const float nx[3], int order, float k,
                                                       float wr) {
        KVals<float> acc;
        acc.G = acc.H = acc.HT = acc.E = cmk(0.f, 0.f);
        const int np = e.nv == 3 ? tri_count(order) : quad_count(order);
        for (int g = 0; g < np; ++g) {
            float s, t, w;
            if (e.nv == 3) {
                const int o = tri_offset(order) + g;
                s = c_trif[o][0]; t = c_trif[o][1]; w = c_trif[o][2];
            } else {
                const int a = g / order, b = g - a * order;
                s = c_glxf[order][a]; t = c_glxf[order][b];
                w = c_glwf[order][a] * c_glwf[order][b];
            }
            QPoint<float> q;
            map_point(e, s, t, w, q);
            KVals<float> v = kernel_values(q, nx, k, wr);
            acc.G += v.G; acc.H += v.H; acc.HT += v.HT; acc.E += v.E;
        }
        return acc;
    }
};

template <typename T>
__device__ __forceinline__ cplx<T> col_adm(const DevFreq &f, int j, int bc) {
    if (bc != 2 || f.adm == nullptr) return {T(0), T(0)};
    cplx<double> a = ld_c(f.adm, j);
    return {(T)a.re, (T)a.im};
}

// ------------------------------------------------------------ near list
// Pairs (row i, column j) that NumCalc integrates with subdivision (level-0
// ratio distance/sqrt(area) < 1.3, exact FP64 test) plus the self pairs.
// Depends on the geometry only, so it is built once per mesh.  Pass 1
// (list == nullptr) counts, pass 2 fills; warp-aggregated atomics.
__global__ void __launch_bounds__(256) k_near_list(DevMeshView mv, int2 *list, unsigned long long *count) {
    const DevMesh m = to_dev(mv);
    const int lane = threadIdx.x, n = m.n;
    const int i = blockIdx.y * 8 + threadIdx.y;
    const int j = blockIdx.x * 32 + lane;
    if (i >= n) return;
    bool near = false;
    if (j < n) {
        if (j == i) near = true;
        else {
            const float d0 = (m.chi[j] - m.chi[i]) + (m.clo[j] - m.clo[i]);
            const float d1 = (m.chi[n + j] - m.chi[n + i]) + (m.clo[n + j] - m.clo[n + i]);
            const float d2 = (m.chi[2 * n + j] - m.chi[2 * n + i]) + (m.clo[2 * n + j] - m.clo[2 * n + i]);
            const float rf = sqrtf(d0 * d0 + d1 * d1 + d2 * d2) * m.isqa32[j];
            if (rf <= 1.3f * (1.0f + 1e-4f)) {
                const double x[3] = {m.c64[i], m.c64[n + i], m.c64[2 * n + i]};
                near = ratio0_exact(m, j, x) < kTolf;
            }
        }
    }
    const unsigned mask = __ballot_sync(0xffffffffu, near);
    if (!mask) return;
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(count, (unsigned long long)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (near && list) list[base + __popc(mask & ((1u << lane) - 1u))] = make_int2(i, j);
}

// ------------------------------------------------------------ regular pairs
// Regular (not subdivided) pairs: block of 8 warps, every warp 4 rows x 32
// columns, one column per lane.  The column element is loaded once per lane
// and reused for its 4 rows; entries go out as coalesced row segments.  Near
// and self pairs are skipped here and written by k_near.
constexpr int kRowsPerThread = 4;

template <typename T>
__global__ void __launch_bounds__(256, 3) k_far(DevMeshView mv, DevFreq f, typename Vec2<T>::type *__restrict__ A,
                                             size_t lda) {
    const DevMesh m = to_dev(mv);
    const int lane = threadIdx.x, n = m.n;
    const int i0 = (blockIdx.y * 8 + threadIdx.y) * kRowsPerThread;
    const int j = blockIdx.x * 32 + lane;
    if (i0 >= n || j >= n) return;
    Phys<T> PT;
    if constexpr (std::is_same<T, double>::value) PT = {f.k, f.wr, f.tao, f.beta_im};
    else PT = {f.kf, f.wrf, f.taof, f.beta_imf};
    const int bcj = f.bc_type ? f.bc_type[j] : 0;
    const cplx<T> admj = col_adm<T>(f, j, bcj);
    if constexpr (std::is_same<T, double>::value) {
        Elem64 e;
        load_elem64(m, j, e);
        for (int r = 0; r < kRowsPerThread; ++r) {
            const int i = i0 + r;
            if (i >= n) break;
            if (i == j) continue;
            const double x64[3] = {m.c64[i], m.c64[n + i], m.c64[2 * n + i]};
            const double rd = ratio0_exact(m, j, x64);
            if (rd < kTolf) continue;
            const double nx64[3] = {m.n64[i], m.n64[n + i], m.n64[2 * n + i]};
            KVals<double> v = FarPair<double>::run(e, x64, nx64, gauss_order(rd), f.k, f.wr);
            const cplx<double> val = combine_entry(v, bcj, admj, PT);
            A[(size_t)i * lda + j] = make_double2(val.re, val.im);
        }
    } else {
        Elem32 e;
        const float zero[3] = {0.f, 0.f, 0.f};
        load_elem32(m, j, zero, zero, e);
        const float cjh[3] = {m.chi[j], m.chi[n + j], m.chi[2 * n + j]};
        const float cjl[3] = {m.clo[j], m.clo[n + j], m.clo[2 * n + j]};
        const float isq = m.isqa32[j];
        for (int r = 0; r < kRowsPerThread; ++r) {
            const int i = i0 + r;
            if (i >= n) break;
            if (i == j) continue;
            for (int k = 0; k < 3; ++k) e.D[k] = (cjh[k] - m.chi[k * n + i]) + (cjl[k] - m.clo[k * n + i]);
            const float rf = sqrtf(e.D[0] * e.D[0] + e.D[1] * e.D[1] + e.D[2] * e.D[2]) * isq;
            bool near = false;
            int order = 2;
            if (!classify_fast(rf, near, order)) {
                const double x64[3] = {m.c64[i], m.c64[n + i], m.c64[2 * n + i]};
                const double rd = ratio0_exact(m, j, x64);
                near = rd < kTolf;
                if (!near) order = gauss_order(rd);
            }
            if (near) continue;
            const float nx[3] = {m.n32[i], m.n32[n + i], m.n32[2 * n + i]};
            KVals<float> v = FarPair<float>::run(e, nx, order, PT.k, PT.wr);
            const cplx<float> val = combine_entry(v, bcj, admj, PT);
            A[(size_t)i * lda + j] = make_float2(val.re, val.im);
        }
    }
}

// ------------------------------------------------------------ near pairs
// One warp per entry of the near list: the self pair by warp_singular (FP64,
// plus NumCalc's free term), subdivided pairs by warp_subdivide with the
// kernel arithmetic in T.
template <typename T>
__global__ void __launch_bounds__(256) k_near(DevMeshView mv, DevFreq f, const int2 *__restrict__ list, long long count,
                                              typename Vec2<T>::type *__restrict__ A, size_t lda, int *status) {
    __shared__ WarpScratch ws_all[8];
    const DevMesh m = to_dev(mv);
    const int lane = threadIdx.x, n = m.n;
    const long long idx = (long long)blockIdx.x * 8 + threadIdx.y;
    if (idx >= count) return;
    WarpScratch &ws = ws_all[threadIdx.y];
    const int2 ij = list[idx];
    const int i = ij.x, j = ij.y;
    const double x64[3] = {m.c64[i], m.c64[n + i], m.c64[2 * n + i]};
    const double nx64[3] = {m.n64[i], m.n64[n + i], m.n64[2 * n + i]};
    Phys<double> P{f.k, f.wr, f.tao, f.beta_im};
    Phys<T> PT{(T)f.k, (T)f.wr, (T)f.tao, (T)f.beta_im};
    const int bcj = f.bc_type ? f.bc_type[j] : 0;
    Elem64 e;
    load_elem64(m, j, e);
    cplx<T> entry;
    int err = kDevOk;
    if (i == j) {
        SingOut so = warp_singular(e, x64, nx64, P, 0, nullptr);
        cplx<double> a = combine_entry(so.v, bcj, col_adm<double>(f, j, bcj), P);
        // free term, NC_EquationSystem.cpp:220-231
        const cplx<double> beta = {0.0, P.beta_im};
        if (bcj == 1) a += beta * (-(0.5 * P.tao));
        else a += (col_adm<double>(f, j, bcj) * beta - cplx<double>{1.0, 0.0}) * 0.5;
        entry = {(T)a.re, (T)a.im};
    } else if constexpr (std::is_same<T, double>::value) {
        AsmSink<double> sink;
        sink.e = &e; sink.x = x64; sink.nx = nx64; sink.k = f.k; sink.wr = f.wr;
        sink.init();
        err = warp_subdivide(e, m.area64[j], x64, ws, sink);
        KVals<double> v = sink.reduce();
        entry = combine_entry(v, bcj, col_adm<double>(f, j, bcj), PT);
    } else {
        const float xhi[3] = {m.chi[i], m.chi[n + i], m.chi[2 * n + i]};
        const float xlo[3] = {m.clo[i], m.clo[n + i], m.clo[2 * n + i]};
        const float nx32[3] = {(float)nx64[0], (float)nx64[1], (float)nx64[2]};
        Elem32 e32;
        load_elem32(m, j, xhi, xlo, e32);
        AsmSink<float> sink;
        sink.e = &e32; sink.nx = nx32; sink.k = PT.k; sink.wr = PT.wr;
        sink.init();
        err = warp_subdivide(e, m.area64[j], x64, ws, sink);
        KVals<float> v = sink.reduce();
        entry = combine_entry(v, bcj, col_adm<float>(f, j, bcj), PT);
    }
    if (lane == 0) {
        typename Vec2<T>::type o;
        o.x = entry.re;
        o.y = entry.im;
        A[(size_t)i * lda + j] = o;
        if (err != kDevOk) atomicMax(status, err);
    }
}

// Incident waves at a collocation point (NC_IncidentWaveRHS,
// NC_EquationSystem.cpp:1731-1812), without symmetry planes.
__device__ cplx<double> incident_rhs(const DevFreq &f, const double x[3], const double nx[3]) {
    cplx<double> zrc = {0.0, 0.0};
    const cplx<double> bt = {0.0, f.beta_im * f.tao};
    for (int s = 0; s < f.n_plane; ++s) {
        const double *d = f.pw_dir + 3 * s;
        const cplx<double> amp = ld_c(f.pw_amp, s);
        const double ph = (d[0] * x[0] + d[1] * x[1] + d[2] * x[2]) * f.wr;
        double sn, cs;
        sincos(ph, &sn, &cs);
        const cplx<double> zg = cplx<double>{cs, sn} * amp;
        const double re1 = f.wr * (d[0] * nx[0] + d[1] * nx[1] + d[2] * nx[2]);
        const cplx<double> zv = {-zg.im * re1, zg.re * re1};
        zrc -= zg + zv * bt;
    }
    for (int s = 0; s < f.n_point; ++s) {
        const double *p = f.ps_xyz + 3 * s;
        const cplx<double> amp = ld_c(f.ps_amp, s);
        double d[3] = {x[0] - p[0], x[1] - p[1], x[2] - p[2]};
        const double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        d[0] /= r; d[1] /= r; d[2] /= r;
        double sn, cs;
        sincos(f.wr * r, &sn, &cs);
        const double re2 = 1.0 / kPI4 / r;
        const cplx<double> zg = cplx<double>{cs * re2, sn * re2} * amp;
        const double re1 = d[0] * nx[0] + d[1] * nx[1] + d[2] * nx[2];
        const cplx<double> zv = cplx<double>{-re1 / r, f.wr * re1} * zg;
        zrc -= zg + zv * bt;
    }
    return zrc;
}

// Right-hand side, one warp per row (FP64): free term of the prescribed value
// (NC_EquationSystem.cpp:233-244), incident waves, and the columns whose
// prescribed values are nonzero (Zrsintel[4], NC_EquationSystem.cpp:188-198).
__global__ void __launch_bounds__(256) k_rhs(DevMeshView mv, DevFreq f, double2 *b, int *status) {
    __shared__ WarpScratch ws_all[8];
    const DevMesh m = to_dev(mv);
    const int lane = threadIdx.x, w = threadIdx.y;
    const int n = m.n;
    const int i = blockIdx.x * 8 + w;
    if (i >= n) return;
    WarpScratch &ws = ws_all[w];
    const double x[3] = {m.c64[i], m.c64[n + i], m.c64[2 * n + i]};
    const double nx[3] = {m.n64[i], m.n64[n + i], m.n64[2 * n + i]};
    Phys<double> P{f.k, f.wr, f.tao, f.beta_im};
    const cplx<double> beta = {0.0, f.beta_im};
    cplx<double> z0 = {0.0, 0.0};
    if (lane == 0) {
        const int bci = f.bc_type ? f.bc_type[i] : 0;
        cplx<double> zbvi = {0.0, 0.0};
        const int nv = m.nvert[i];
        if (f.bc_val)
            for (int a = 0; a < nv; ++a) zbvi += ld_c(f.bc_val, a * n + i);
        zbvi = {zbvi.re / (double)nv, zbvi.im / (double)nv};
        if (bci != 1) z0 += ((zbvi * beta) * f.tao) * 0.5;
        else z0 += (zbvi * f.tao) * 0.5;
        if (f.n_plane + f.n_point > 0) z0 += incident_rhs(f, x, nx);
    }
    int err = kDevOk;
    for (int c = 0; c < f.n_bc_cols; ++c) {
        const int jc = f.bc_cols[c];
        const int bcj = f.bc_type ? f.bc_type[jc] : 0;
        Elem64 e;
        load_elem64(m, jc, e);
        cplx<double> bc[4];
        for (int a = 0; a < 4; ++a) bc[a] = a < e.nv ? ld_c(f.bc_val, a * n + jc) : cplx<double>{0.0, 0.0};
        cplx<double> contrib;
        if (jc == i) {
            SingOut so = warp_singular(e, x, nx, P, bcj == 1 ? 2 : 1, bc);
            contrib = so.rhs;
        } else {
            RhsSink sink;
            sink.e = &e; sink.x = x; sink.nx = nx; sink.bc = bc; sink.bctype = bcj == 1 ? 1 : 0; sink.P = P;
            sink.init();
            const int rc = warp_subdivide(e, m.area64[jc], x, ws, sink);
            if (rc != kDevOk) err = rc;
            contrib = sink.reduce();
        }
        if (lane == 0) z0 += contrib;
    }
    if (lane == 0) {
        b[i] = make_double2(z0.re, z0.im);
        if (err != kDevOk) atomicMax(status, err);
    }
}

// Element potentials and nodal normal velocities after the solve
// (NC_WriteResultsObjectMesh, NC_PostProcessing.cpp:389-410).
__global__ void k_fields(DevMeshView mv, DevFreq f, const double2 *x, double2 *phi, double2 *vel, int *ivi) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = mv.n;
    if (j >= n) return;
    const int bc = f.bc_type ? f.bc_type[j] : 0;
    const int nv = mv.nvert[j];
    const cplx<double> xj = {x[j].x, x[j].y};
    cplx<double> p, v[4];
    for (int a = 0; a < 4; ++a)
        v[a] = (f.bc_val && a < nv) ? ld_c(f.bc_val, a * n + j) : cplx<double>{0.0, 0.0};
    if (bc == 1) {
        p = v[0];
        for (int a = 0; a < 4; ++a) v[a] = a < nv ? xj : cplx<double>{0.0, 0.0};
    } else {
        p = xj;
        if (bc == 2 && f.adm) {
            const cplx<double> z1 = (xj * ld_c(f.adm, j)) * f.tao;
            for (int a = 0; a < nv; ++a) v[a] -= z1;
        }
    }
    int any = 0;
    for (int a = 0; a < nv; ++a)
        if (sqrt(v[a].re * v[a].re + v[a].im * v[a].im) > kEPSY) any = 1;
    phi[j] = make_double2(p.re, p.im);
    for (int a = 0; a < 4; ++a) vel[a * n + j] = make_double2(v[a].re, v[a].im);
    ivi[j] = any;
}

// Field projection, one warp per point: lanes sweep the elements 32 at a time;
// regular pairs in the lane, subdivided pairs by the whole warp.
template <typename T>
__global__ void __launch_bounds__(256) k_project(DevMeshView mv, DevFreq f, const double2 *phi, const double2 *vel,
                                                 const int *ivi, int npts, const double *pts, double2 *pot,
                                                 double2 *grad, int *status) {
    __shared__ WarpScratch ws_all[8];
    const DevMesh m = to_dev(mv);
    const int lane = threadIdx.x, w = threadIdx.y;
    const int n = m.n;
    const int p = blockIdx.x * 8 + w;
    if (p >= npts) return;
    WarpScratch &ws = ws_all[w];
    const double x64[3] = {pts[3 * p], pts[3 * p + 1], pts[3 * p + 2]};
    float xhi[3], xlo[3];
    for (int k = 0; k < 3; ++k) {
        xhi[k] = (float)x64[k];
        xlo[k] = (float)(x64[k] - (double)xhi[k]);
    }
    ProjAcc<T> acc;
    acc.p = acc.g[0] = acc.g[1] = acc.g[2] = cmk(T(0), T(0));
    const T k = (T)f.k, wr = (T)f.wr;
    int err = kDevOk;
    for (int base = 0; base < n; base += 32) {
        const int j = base + lane;
        const bool valid = j < n;
        bool near = false;
        int order = 2;
        if (valid) {
            cplx<T> ph = {(T)phi[j].x, (T)phi[j].y};
            const bool iv = ivi[j] != 0;
            cplx<T> vl[4];
            for (int a = 0; a < 4; ++a) vl[a] = {(T)vel[a * n + j].x, (T)vel[a * n + j].y};
            if constexpr (std::is_same<T, double>::value) {
                const double rd = ratio0_exact(m, j, x64);
                near = rd < kTolf;
                if (!near) {
                    order = gauss_order(rd);
                    Elem64 e;
                    load_elem64(m, j, e);
                    const int np = e.nv == 3 ? tri_count(order) : quad_count(order);
                    for (int g = 0; g < np; ++g) {
                        double s, t, wq;
                        sub_point(e.nv, order, g, 0.0, 0.0, 1.0, s, t, wq);
                        QPoint<double> q;
                        map_point(e, s, t, x64, wq, q);
                        proj_point(q, ph, vl, e.nv, iv, k, wr, acc);
                    }
                }
            } else {
                Elem32 e;
                load_elem32(m, j, xhi, xlo, e);
                const float dist = sqrtf(e.D[0] * e.D[0] + e.D[1] * e.D[1] + e.D[2] * e.D[2]);
                if (!classify_fast(dist * m.isqa32[j], near, order)) {
                    const double rd = ratio0_exact(m, j, x64);
                    near = rd < kTolf;
                    if (!near) order = gauss_order(rd);
                }
                if (!near) {
                    const int np = e.nv == 3 ? tri_count(order) : quad_count(order);
                    for (int g = 0; g < np; ++g) {
                        float s, t, wq;
                        if (e.nv == 3) {
                            const int o = tri_offset(order) + g;
                            s = c_trif[o][0]; t = c_trif[o][1]; wq = c_trif[o][2];
                        } else {
                            const int a = g / order, b = g - a * order;
                            s = c_glxf[order][a]; t = c_glxf[order][b];
                            wq = c_glwf[order][a] * c_glwf[order][b];
                        }
                        QPoint<float> q;
                        map_point(e, s, t, wq, q);
                        proj_point(q, ph, vl, e.nv, iv, k, wr, acc);
                    }
                }
            }
        }
        unsigned todo = __ballot_sync(0xffffffffu, valid && near);
        while (todo) {
            const int L = __ffs(todo) - 1;
            todo &= todo - 1;
            const int jl = base + L;
            Elem64 e;
            load_elem64(m, jl, e);
            cplx<T> ph = {(T)phi[jl].x, (T)phi[jl].y};
            cplx<T> vl[4];
            for (int a = 0; a < 4; ++a) vl[a] = {(T)vel[a * n + jl].x, (T)vel[a * n + jl].y};
            const bool iv = ivi[jl] != 0;
            ProjAcc<T> r;
            int rc;
            if constexpr (std::is_same<T, double>::value) {
                ProjSink<double> sink;
                sink.e = &e; sink.x = x64; sink.phi = ph; sink.vel = vl; sink.ivi = iv; sink.k = k; sink.wr = wr;
                sink.init();
                rc = warp_subdivide(e, m.area64[jl], x64, ws, sink);
                r = sink.reduce();
            } else {
                Elem32 e32;
                load_elem32(m, jl, xhi, xlo, e32);
                ProjSink<float> sink;
                sink.e = &e32; sink.phi = ph; sink.vel = vl; sink.ivi = iv; sink.k = k; sink.wr = wr;
                sink.init();
                rc = warp_subdivide(e, m.area64[jl], x64, ws, sink);
                r = sink.reduce();
            }
            if (rc != kDevOk) err = rc;
            if (lane == 0) {
                acc.p += r.p;
                for (int kk = 0; kk < 3; ++kk) acc.g[kk] += r.g[kk];
            }
        }
    }
    // FP64 cross-lane reduction
    cplx<double> sp = warp_sum(cplx<double>{(double)acc.p.re, (double)acc.p.im});
    cplx<double> sg[3];
    for (int kk = 0; kk < 3; ++kk) sg[kk] = warp_sum(cplx<double>{(double)acc.g[kk].re, (double)acc.g[kk].im});
    if (lane == 0) {
        if (f.tao != 1.0) {
            sp = sp * f.tao;
            for (int kk = 0; kk < 3; ++kk) sg[kk] = sg[kk] * f.tao;
        }
        // incident field (NC_ContributionIncidentWaves, NC_PostProcessing.cpp:776-866)
        if (f.n_plane || f.n_point) {
            for (int s = 0; s < f.n_plane; ++s) {
                const double *d = f.pw_dir + 3 * s;
                const cplx<double> amp = ld_c(f.pw_amp, s);
                double sn, cs;
                sincos((d[0] * x64[0] + d[1] * x64[1] + d[2] * x64[2]) * f.wr, &sn, &cs);
                const cplx<double> zg = cplx<double>{cs, sn} * amp;
                sp += zg;
                const cplx<double> zv = {-zg.im * f.wr, zg.re * f.wr};
                for (int kk = 0; kk < 3; ++kk) sg[kk] += zv * d[kk];
            }
            for (int s = 0; s < f.n_point; ++s) {
                const double *q = f.ps_xyz + 3 * s;
                const cplx<double> amp = ld_c(f.ps_amp, s);
                double d[3] = {x64[0] - q[0], x64[1] - q[1], x64[2] - q[2]};
                const double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                d[0] /= r; d[1] /= r; d[2] /= r;
                double sn, cs;
                sincos(f.wr * r, &sn, &cs);
                const double re2 = 1.0 / kPI4 / r;
                const cplx<double> zg = cplx<double>{cs * re2, sn * re2} * amp;
                sp += zg;
                const cplx<double> zv = cplx<double>{-1.0 / r, f.wr} * zg;
                for (int kk = 0; kk < 3; ++kk) sg[kk] += zv * d[kk];
            }
        }
        pot[p] = make_double2(sp.re, sp.im);
        if (grad)
            for (int kk = 0; kk < 3; ++kk) grad[3 * p + kk] = make_double2(sg[kk].re, sg[kk].im);
        if (err != kDevOk) atomicMax(status, err);
    }
}

// ---------------------------------------------------------------- tables
// Published Gauss-Legendre and triangle rules at the precision NumCalc
// tabulates them (NC_IntegrationConstants.h:26-49,3729-3865).
const double kGLPos[7][3][2] = {
    {{0, 0}},
    {{0.0, 2.0}},
    {{0.577350269189626, 1.0}},
    {{0.0, 0.888888888888889}, {0.774596669241483, 0.555555555555556}},
    {{0.339981043584856, 0.652145154862546}, {0.861136311594053, 0.347854845137454}},
    {{0.0, 0.568888888888889}, {0.538469310105683, 0.478628670499366}, {0.906179845938664, 0.236926885056189}},
    {{0.238619186083197, 0.467913934572691}, {0.661209386466265, 0.360761573048139}, {0.932469514203152, 0.171324492379170}},
};

const double kTri[24][3] = {
    // Strang-Fix 4 points
    {1.0 / 3.0, 1.0 / 3.0, -27.0 / 96.0}, {0.2, 0.2, 25.0 / 96.0}, {0.6, 0.2, 25.0 / 96.0}, {0.2, 0.6, 25.0 / 96.0},
    // Radon 7 points
    {0.1012865073235, 0.1012865073235, 0.1259391805448 / 2.0},
    {0.7974269853531, 0.1012865073235, 0.1259391805448 / 2.0},
    {0.1012865073235, 0.7974269853531, 0.1259391805448 / 2.0},
    {0.4701420641051, 0.0597158717898, 0.1323941527885 / 2.0},
    {0.4701420641051, 0.4701420641051, 0.1323941527885 / 2.0},
    {0.0597158717898, 0.4701420641051, 0.1323941527885 / 2.0},
    {0.3333333333333, 0.3333333333333, 0.225 / 2.0},
    // 13 points, degree 7
    {0.0651301029022, 0.0651301029022, 0.0533472356088 / 2.0},
    {0.8697397941956, 0.0651301029022, 0.0533472356088 / 2.0},
    {0.0651301029022, 0.8697397941956, 0.0533472356088 / 2.0},
    {0.3128654960049, 0.0486903154253, 0.0771137608903 / 2.0},
    {0.6384441885698, 0.3128654960049, 0.0771137608903 / 2.0},
    {0.0486903154253, 0.6384441885698, 0.0771137608903 / 2.0},
    {0.6384441885698, 0.0486903154253, 0.0771137608903 / 2.0},
    {0.3128654960049, 0.6384441885698, 0.0771137608903 / 2.0},
    {0.0486903154253, 0.3128654960049, 0.0771137608903 / 2.0},
    {0.2603459660790, 0.2603459660790, 0.1756152574332 / 2.0},
    {0.4793080678419, 0.2603459660790, 0.1756152574332 / 2.0},
    {0.2603459660790, 0.4793080678419, 0.1756152574332 / 2.0},
    {0.3333333333333, 0.3333333333333, -0.1495700444677 / 2.0},
};

// Host copy of NumCalc's order test (NC_Macros.h:44-50) for the thresholds.
bool order_ok_host(int m, double ratdis) {
    const double disfac = 0.5 / ratdis;
    double eg = 32.0, eh = 64.0 * (2.0 * (double)m + 1.0), ee = 128.0 * ((double)m + 1.0) * (2.0 * (double)m + 1.0);
    for (int q = 0; q < 2 * m + 1; ++q) eg *= disfac;
    for (int q = 0; q < 2 * m + 2; ++q) eh *= disfac;
    for (int q = 0; q < 2 * m + 3; ++q) ee *= disfac;
    return ee < 0.001 && eh < 0.001 && eg < 0.001;
}

double order_threshold(int m) {
    // bisection over the ordered bit patterns of positive doubles
    double lo = 0.5, hi = 1000.0;  // order_ok false at lo, true at hi
    uint64_t a, b;
    memcpy(&a, &lo, 8);
    memcpy(&b, &hi, 8);
    while (b - a > 1) {
        uint64_t c = a + (b - a) / 2;
        double mid;
        memcpy(&mid, &c, 8);
        if (order_ok_host(m, mid)) b = c; else a = c;
    }
    double t;
    memcpy(&t, &b, 8);
    return t;
}

}  // namespace

cudaError_t init_device_tables() {
    QuadTables q;
    memset(&q, 0, sizeof(q));
    float trif[24][3], glxf[7][6], glwf[7][6];
    for (int i = 0; i < 24; ++i)
        for (int k = 0; k < 3; ++k) { q.tri[i][k] = kTri[i][k]; trif[i][k] = (float)kTri[i][k]; }
    for (int n = 1; n <= 6; ++n) {
        const int h = n / 2;
        double x[6] = {0}, w[6] = {0};
        if (n % 2) {
            x[h] = kGLPos[n][0][0]; w[h] = kGLPos[n][0][1];
            for (int i = 1; i <= h; ++i) {
                x[h + i] = kGLPos[n][i][0]; x[h - i] = -kGLPos[n][i][0];
                w[h + i] = w[h - i] = kGLPos[n][i][1];
            }
        } else {
            for (int i = 0; i < h; ++i) {
                x[h + i] = kGLPos[n][i][0]; x[h - 1 - i] = -kGLPos[n][i][0];
                w[h + i] = w[h - 1 - i] = kGLPos[n][i][1];
            }
        }
        for (int i = 0; i < 6; ++i) {
            q.glx[n][i] = x[i]; q.glw[n][i] = w[i];
            glxf[n][i] = (float)x[i]; glwf[n][i] = (float)w[i];
        }
    }
    for (int i = 0; i < 6; ++i) { glxf[0][i] = glwf[0][i] = 0.f; }
    for (int m = 2; m <= 5; ++m) {
        q.order_thr[m] = order_threshold(m);
        q.order_thrf[m] = (float)q.order_thr[m];
    }
    cudaError_t e = cudaMemcpyToSymbol(c_quad, &q, sizeof(q));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_trif, trif, sizeof(trif));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_glxf, glxf, sizeof(glxf));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_glwf, glwf, sizeof(glwf));
    return e;
}

cudaError_t launch_near_list(const DevMeshView &m, int2 *list, unsigned long long *count, cudaStream_t st) {
    dim3 block(32, 8), grid((m.n + 31) / 32, (m.n + 7) / 8);
    count_launches(1);
    k_near_list<<<grid, block, 0, st>>>(m, list, count);
    return cudaGetLastError();
}

cudaError_t launch_assemble(const DevMeshView &m, const DevFreq &f, int prec, void *A, size_t lda,
                            const int2 *near_list, long long n_near, int *status, cudaStream_t st) {
    dim3 block(32, 8), grid((m.n + 31) / 32, (m.n + 8 * kRowsPerThread - 1) / (8 * kRowsPerThread));
    const int nblk = (int)((n_near + 7) / 8);
    count_launches(2);
    if (prec == 0) {
        k_far<double><<<grid, block, 0, st>>>(m, f, (double2 *)A, lda);
        if (nblk) k_near<double><<<nblk, block, 0, st>>>(m, f, near_list, n_near, (double2 *)A, lda, status);
    } else {
        k_far<float><<<grid, block, 0, st>>>(m, f, (float2 *)A, lda);
        if (nblk) k_near<float><<<nblk, block, 0, st>>>(m, f, near_list, n_near, (float2 *)A, lda, status);
    }
    return cudaGetLastError();
}

cudaError_t launch_rhs(const DevMeshView &m, const DevFreq &f, double *b, int *status, cudaStream_t st) {
    dim3 block(32, 8), grid((m.n + 7) / 8);
    count_launches(1);
    k_rhs<<<grid, block, 0, st>>>(m, f, (double2 *)b, status);
    return cudaGetLastError();
}

cudaError_t launch_fields(const DevMeshView &m, const DevFreq &f, const double *x, double *phi, double *vel,
                          int *ivi, cudaStream_t st) {
    count_launches(1);
    k_fields<<<(m.n + 255) / 256, 256, 0, st>>>(m, f, (const double2 *)x, (double2 *)phi, (double2 *)vel, ivi);
    return cudaGetLastError();
}

cudaError_t launch_project(const DevMeshView &m, const DevFreq &f, int prec, const double *phi, const double *vel,
                           const int *ivi, int npts, const double *pts, double *pot, double *grad, int *status,
                           cudaStream_t st) {
    if (npts <= 0) return cudaSuccess;
    dim3 block(32, 8), grid((npts + 7) / 8);
    count_launches(1);
    if (prec == 0)
        k_project<double><<<grid, block, 0, st>>>(m, f, (const double2 *)phi, (const double2 *)vel, ivi, npts, pts,
                                                  (double2 *)pot, (double2 *)grad, status);
    else
        k_project<float><<<grid, block, 0, st>>>(m, f, (const double2 *)phi, (const double2 *)vel, ivi, npts, pts,
                                                 (double2 *)pot, (double2 *)grad, status);
    return cudaGetLastError();
}

}  // namespace bem
