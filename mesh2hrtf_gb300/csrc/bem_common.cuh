// bem_common.cuh - device-side building blocks shared by the assembly and
// projection kernels: complex arithmetic, quadrature tables, the element
// tables of a mesh, the reference's subdivision rule, and the warp-cooperative
// integration of one (point, element) pair.
//
// Precision scheme (see bem_gb300.h, bem_precision): every *decision* that
// selects a quadrature (subdivide or not, Gauss order, subelement origin) is
// taken in FP64 with unfused operations, exactly as NumCalc's x86 build
// takes it, so both precisions integrate with the reference's quadrature.
// The kernel arithmetic runs in T = double (plain path) or T = float (mixed
// path); singular self-element integrals always run in FP64.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "bem_internal.h"

namespace bem {

constexpr double kPI4 = 12.566370614359172944;   // 4 pi, NC_ConstantsVariables.h:66
constexpr double kEPSY = 1.0e-14;                // NC_ConstantsVariables.h:68
constexpr int kMSBE = 220;                       // max subelements, NC_ConstantsVariables.h:63
constexpr int kMaxLevelSub = 60;                 // 15 splits x 4 children per level
constexpr int kMaxLevel = 22;                    // deepest level with exact float coordinates
constexpr double kTolf = 1.3;                    // subdivision ratio, NC_3dFunctions.cpp:599

// error codes written to the device status word
enum DevErr : int { kDevOk = 0, kDevSplitLimit = 1, kDevSubLimit = 2 };

// ------------------------------------------------------------ complex
template <typename T> struct cplx { T re, im; };
template <typename T> __device__ __forceinline__ cplx<T> cmk(T r, T i) { return {r, i}; }
template <typename T> __device__ __forceinline__ cplx<T> operator+(cplx<T> a, cplx<T> b) { return {a.re + b.re, a.im + b.im}; }
template <typename T> __device__ __forceinline__ cplx<T> operator-(cplx<T> a, cplx<T> b) { return {a.re - b.re, a.im - b.im}; }
template <typename T> __device__ __forceinline__ cplx<T> operator*(cplx<T> a, cplx<T> b) {
    return {a.re * b.re - a.im * b.im, a.im * b.re + a.re * b.im};
}
template <typename T> __device__ __forceinline__ cplx<T> operator*(cplx<T> a, T s) { return {a.re * s, a.im * s}; }
template <typename T> __device__ __forceinline__ void operator+=(cplx<T> &a, cplx<T> b) { a.re += b.re; a.im += b.im; }
template <typename T> __device__ __forceinline__ void operator-=(cplx<T> &a, cplx<T> b) { a.re -= b.re; a.im -= b.im; }

template <typename T> __device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
template <typename T> __device__ __forceinline__ cplx<T> warp_sum(cplx<T> v) {
    return {warp_sum(v.re), warp_sum(v.im)};
}

// The hardware approximations (PTX sin/cos/rsqrt.approx) with denormal
// inputs flushed to zero: without .ftz the compiler wraps each in a
// denormal test and rescaling (the library build keeps IEEE denormals).
// Normal inputs give the same results as the non-ftz forms.
__device__ __forceinline__ float sin_approx(float x) {
    float y;
    asm("sin.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float cos_approx(float x) {
    float y;
    asm("cos.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
// 1/sqrt(x) for squared distances (never denormal: >= 1e-12 m^2 here)
__device__ __forceinline__ float rsqrt_approx(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// sin and cos of a float phase k*r: Cody & Waite reduction by 2 pi (2 pi
// split into two floats, x / 2 pi rounded with the 1.5 * 2^23 shifter, which
// needs no float-to-integer conversion: on GB300 those issue on the narrow
// FP64 pipe), then the hardware approximations, accurate to about 2^-21
// absolute on [-pi, pi].  The mixed-precision path's error budget is 1e-4
// against FP64; this keeps it near 3e-6.
__device__ __forceinline__ void phase_sincos(float x, float *s, float *c) {
    const float sh = fmaf(x, 0.159154943f, 12582912.0f);   // 1 / (2 pi), 1.5 * 2^23
    const float q = sh - 12582912.0f;
    float r = fmaf(q, -6.28318548202514648f, x);
    r = fmaf(q, 1.74845553146951e-07f, r);
    *s = sin_approx(r);
    *c = cos_approx(r);
}

__device__ __forceinline__ void sincos_t(double x, double *s, double *c) { sincos(x, s, c); }
__device__ __forceinline__ void sincos_t(float x, float *s, float *c) { phase_sincos(x, s, c); }
__device__ __forceinline__ double sqrt_t(double x) { return sqrt(x); }
__device__ __forceinline__ float sqrt_t(float x) { return sqrtf(x); }

// ------------------------------------------------------------ quadrature
// Triangle rules on the (1,0),(0,1),(0,0) reference triangle (weights sum to
// 0.5): Strang-Fix 4-point (order 2), Radon 7-point (order 3), 13-point
// degree-7 rule (orders 4..7), with the values NumCalc tabulates
// (NC_IntegrationConstants.h:3729-3865).  Stored back to back: 4 + 7 + 13.
// Gauss-Legendre 1..6 points on [-1, 1], ascending, as NumCalc's BLGauCooWe
// lays them out (NC_CommonFunctions.cpp:412-1063).
struct QuadTables {
    double tri[24][3];
    double glx[7][6];
    double glw[7][6];
    // orders 2..5: smallest ratio (distance / sqrt(area)) for which NumCalc's
    // error estimates (NC_Macros.h:44-50) accept that order; below thr[5] the
    // order is 6.  Computed on the host by bisection over doubles.
    double order_thr[8];
    float order_thrf[8];
    // squared ratio beyond which the float test alone gives order 2 (the
    // order-2 threshold with a 3e-5 margin): skips the square root and the
    // threshold scan for most regular pairs
    float far2_sq;
};
// Defined here: exactly one translation unit (bem_kernels.cu) includes this
// header.
__constant__ QuadTables c_quad;
__constant__ float c_trif[24][3];
// The 4-point rule's (s - 1/3, t - 1/3, 2 (s - 1/3), 2 (t - 1/3)): operands of
// the expanded squared distance of the order-2 far pairs.
__constant__ float c_far4[4][4];
__constant__ float c_glxf[7][6];
__constant__ float c_glwf[7][6];
// local node coordinates of 6-/8-noded parents, NC_Arrays.h:126-129
__constant__ double c_csi8[8] = {1.0, -1.0, -1.0, 1.0, 0.0, -1.0, 0.0, 1.0};
__constant__ double c_eta8[8] = {1.0, 1.0, -1.0, -1.0, 1.0, 0.0, -1.0, 0.0};
__constant__ double c_csi6[6] = {1.0, 0.0, 0.0, 0.5, 0.0, 0.5};
__constant__ double c_eta6[6] = {0.0, 1.0, 0.0, 0.5, 0.5, 0.0};
// the same corner and mid-side points in float (FP32 singular rule)
__constant__ float c_csi8f[8] = {1.f, -1.f, -1.f, 1.f, 0.f, -1.f, 0.f, 1.f};
__constant__ float c_eta8f[8] = {1.f, 1.f, -1.f, -1.f, 1.f, 0.f, -1.f, 0.f};
__constant__ float c_csi6f[6] = {1.f, 0.f, 0.f, 0.5f, 0.f, 0.5f};
__constant__ float c_eta6f[6] = {0.f, 1.f, 0.f, 0.5f, 0.5f, 0.f};

__host__ __device__ constexpr int tri_offset(int order) { return order <= 2 ? 0 : (order == 3 ? 4 : 11); }
__host__ __device__ constexpr int tri_count(int order) { return order <= 2 ? 4 : (order == 3 ? 7 : 13); }
__host__ __device__ constexpr int quad_count(int order) { return order * order; }

// NumCalc's order choice for a subelement at distance ratio `ratdis`
// (NC_3dFunctions.cpp:760-773 with NC_Macros.h:44-50), evaluated exactly: the
// multiplications are plain products (no fusion possible), so the IEEE result
// equals the x86 reference's.
__device__ __forceinline__ int gauss_order_exact(double ratdis) {
    double disfac = 0.5 / ratdis;
    for (int m = 2; m <= 6; ++m) {
        double eg = 32.0, eh = 64.0 * (2.0 * (double)m + 1.0),
               ee = 128.0 * ((double)m + 1.0) * (2.0 * (double)m + 1.0);
        for (int q = 0; q < 2 * m + 1; ++q) eg = __dmul_rn(eg, disfac);
        for (int q = 0; q < 2 * m + 2; ++q) eh = __dmul_rn(eh, disfac);
        for (int q = 0; q < 2 * m + 3; ++q) ee = __dmul_rn(ee, disfac);
        if (ee < 0.001 && eh < 0.001 && eg < 0.001) return m;
    }
    return 6;
}

// Same decision from precomputed thresholds, falling back to the exact loop
// within a few ulps of a threshold.
__device__ __forceinline__ int gauss_order(double ratdis) {
#pragma unroll
    for (int m = 2; m <= 5; ++m) {
        double t = c_quad.order_thr[m];
        if (fabs(ratdis - t) <= 1e-13 * t) return gauss_order_exact(ratdis);
        if (ratdis >= t) return m;
    }
    return 6;
}

// Approximate decision (split, Gauss order) in float; returns false if the ratio lies too
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

// ------------------------------------------------------------ mesh tables
// Device element tables, structure of arrays (index [row * n + element]).
struct DevMesh {
    int n;
    const int *nvert;       // 3 or 4
    const double *v64;      // 12 rows: vertex a (0..3), coordinate k -> row 3a+k
    const double *c64;      // 3 rows: centre (NumCalc's centel)
    const double *n64;      // 3 rows: unit normal at the centre (elenor[.][0..2])
    const double *area64;   // areael
    const double *sqa64;    // sqrt(areael), correctly rounded
    const float *chi;       // 3 rows: centre, high float part
    const float *clo;       // 3 rows: centre - float(high), low part
    const float *t32;       // 10 rows (triangles): a = P0-P2, b = P1-P2, n, J
    const float *q32;       // 12 rows (quads): vertex offsets from the centre
    const float *isqa32;    // 1 / sqrt(areael) in float (approximate ratios)
    const float *n32;       // 3 rows: centre normal in float
    const float4 *row4;     // [n][3]: (chi, 0), (clo, 0), (n32, 0): a collocation
                            // row's data in three 16-byte loads
    DevSym sym;             // symmetry-plane images (sym.nref = 1: none)
};

// Element tables of image kref of every element (kref = 0: the mesh).  The
// images share nvert, areas and 1/sqrt(area) with their elements; their
// v64/c64/chi/clo/t32/q32 rows hold the mirrored vertices in the
// reference's node order and the centre NumCalc's subdivision computes from
// them (global coordinates at the local centre, NC_3dFunctions.cpp:625-640).
// n64/n32 stay the mesh's own: they are read for collocation rows only.
__device__ __forceinline__ DevMesh image_mesh(const DevMesh &m, int kref) {
    if (kref == 0) return m;
    DevMesh r = m;
    const size_t n = (size_t)m.n, k = (size_t)(kref - 1);
    r.v64 = m.sym.v64 + k * 12 * n;
    r.c64 = m.sym.c64 + k * 3 * n;
    r.chi = m.sym.chi + k * 3 * n;
    r.clo = m.sym.clo + k * 3 * n;
    r.t32 = m.sym.t32 + k * 10 * n;
    r.q32 = m.sym.q32 + k * 12 * n;
    return r;
}

// Reflection factor (+1 / -1) of image kref.
__device__ __forceinline__ bool image_negated(const DevMesh &m, int kref) { return (m.sym.rneg >> kref) & 1u; }

// Node a of image kref holds the data of the element's node image_node(a):
// every reflection swaps nodes 0/1, and 2/3 of quadrilaterals
// (NC_3dFunctions.cpp:427-451).
__device__ __forceinline__ int image_node(int a, int kref, int nv) {
    return ((kref & 1) && (a < 2 || nv == 4)) ? (a ^ 1) : a;
}

// One element in registers (FP64), for decisions and the FP64 arithmetic.
struct Elem64 {
    int nv;
    double p[4][3];
};

__device__ __forceinline__ void load_elem64(const DevMesh &m, int j, Elem64 &e) {
    e.nv = m.nvert[j];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int k = 0; k < 3; ++k) e.p[a][k] = (a < e.nv) ? m.v64[(3 * a + k) * m.n + j] : 0.0;
}

// Shape functions and global point, NC_ComputeGlobalCoordinates
// (NC_3dFunctions.cpp:95-129), unfused so that decisions match the reference.
__device__ __forceinline__ void global_point_exact(const Elem64 &e, double s, double t, double x[3]) {
    double sh[4];
    if (e.nv == 3) {
        sh[0] = s; sh[1] = t; sh[2] = __dsub_rn(__dsub_rn(1.0, s), t); sh[3] = 0.0;
    } else {
        double s1 = __dmul_rn(0.25, __dadd_rn(s, 1.0)), s2 = __dmul_rn(0.25, __dsub_rn(s, 1.0));
        double t1 = __dadd_rn(t, 1.0), t2 = __dsub_rn(t, 1.0);
        sh[0] = __dmul_rn(s1, t1); sh[1] = -__dmul_rn(s2, t1);
        sh[2] = __dmul_rn(s2, t2); sh[3] = -__dmul_rn(s1, t2);
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        double acc = 0.0;
        for (int a = 0; a < e.nv; ++a) acc = __dadd_rn(acc, __dmul_rn(sh[a], e.p[a][k]));
        x[k] = acc;
    }
}

__device__ __forceinline__ double dist_exact(const double a[3], const double b[3]) {
    double d0 = __dsub_rn(a[0], b[0]), d1 = __dsub_rn(a[1], b[1]), d2 = __dsub_rn(a[2], b[2]);
    double s = __dadd_rn(__dadd_rn(__dadd_rn(0.0, __dmul_rn(d0, d0)), __dmul_rn(d1, d1)), __dmul_rn(d2, d2));
    return __dsqrt_rn(s);
}

// Level-0 ratio of NC_GenerateSubelements for element j seen from x: the
// whole-element centre is NumCalc's centel and the area its areael.
__device__ __forceinline__ double ratio0_exact(const DevMesh &m, int j, const double x[3]) {
    double c[3] = {m.c64[j], m.c64[m.n + j], m.c64[2 * m.n + j]};
    return __ddiv_rn(dist_exact(c, x), m.sqa64[j]);
}

// ------------------------------------------------------------ pair sinks
// What a quadrature point contributes is decided by a sink; the warp-level
// integration below is shared by assembly (AsmSink), the right-hand side
// (RhsSink) and the field projection (ProjSink).

// Geometry of one quadrature point handed to the sinks.
template <typename T> struct QPoint {
    T d[3];    // y - x
    T r;       // |y - x|
    T ir;      // 1 / r
    T ny[3];   // unit normal at y
    T wj;      // weight * Jacobian
    T sh[4];   // shape functions at y (for interpolating nodal data)
};

// Map local coordinates (s, t) of element j to a quadrature point, FP64.
__device__ __forceinline__ void map_point(const Elem64 &e, double s, double t, const double x[3],
                                          double w, QPoint<double> &q) {
    double sh[4], ds[4], dt[4];
    if (e.nv == 3) {
        sh[0] = s; sh[1] = t; sh[2] = 1.0 - s - t; sh[3] = 0.0;
        ds[0] = 1.0; ds[1] = 0.0; ds[2] = -1.0; ds[3] = 0.0;
        dt[0] = 0.0; dt[1] = 1.0; dt[2] = -1.0; dt[3] = 0.0;
    } else {
        double s1 = 0.25 * (s + 1.0), s2 = 0.25 * (s - 1.0), t1 = t + 1.0, t2 = t - 1.0;
        sh[0] = s1 * t1; sh[1] = -s2 * t1; sh[2] = s2 * t2; sh[3] = -s1 * t2;
        ds[0] = 0.25 * (t + 1.0); ds[2] = 0.25 * (t - 1.0); ds[1] = -ds[0]; ds[3] = -ds[2];
        dt[0] = 0.25 * (s + 1.0); dt[2] = 0.25 * (s - 1.0); dt[1] = -dt[2]; dt[3] = -dt[0];
    }
    double y[3], dxs[3], dxt[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        y[k] = 0.0; dxs[k] = 0.0; dxt[k] = 0.0;
        for (int a = 0; a < e.nv; ++a) {
            y[k] += sh[a] * e.p[a][k];
            dxs[k] += ds[a] * e.p[a][k];
            dxt[k] += dt[a] * e.p[a][k];
        }
    }
    double nx = dxs[1] * dxt[2] - dxt[1] * dxs[2];
    double ny = dxs[2] * dxt[0] - dxt[2] * dxs[0];
    double nz = dxs[0] * dxt[1] - dxt[0] * dxs[1];
    double len = sqrt(nx * nx + ny * ny + nz * nz);
    q.ny[0] = nx / len; q.ny[1] = ny / len; q.ny[2] = nz / len;
    q.wj = w * len;
#pragma unroll
    for (int k = 0; k < 3; ++k) q.d[k] = y[k] - x[k];
    q.r = sqrt(q.d[0] * q.d[0] + q.d[1] * q.d[1] + q.d[2] * q.d[2]);
    q.ir = 1.0 / q.r;
#pragma unroll
    for (int a = 0; a < 4; ++a) q.sh[a] = sh[a];
}

// FP32 element data relative to its centre, and the centre-to-point offset
// D = c_j - x in double-float form (exact for nearby points).
struct Elem32 {
    int nv;
    float D[3];       // centre of j minus the field/collocation point
    float a[3], b[3]; // triangles: P0 - P2, P1 - P2
    float n[3];       // triangles: unit normal
    float J;          // triangles: Jacobian (2 * area)
    float q[4][3];    // quads: vertex offsets from the centre
};

__device__ __forceinline__ void load_elem32(const DevMesh &m, int j, const float xhi[3],
                                            const float xlo[3], Elem32 &e) {
    e.nv = m.nvert[j];
#pragma unroll
    for (int k = 0; k < 3; ++k)
        e.D[k] = (m.chi[k * m.n + j] - xhi[k]) + (m.clo[k * m.n + j] - xlo[k]);
    if (e.nv == 3) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            e.a[k] = m.t32[k * m.n + j];
            e.b[k] = m.t32[(3 + k) * m.n + j];
            e.n[k] = m.t32[(6 + k) * m.n + j];
        }
        e.J = m.t32[9 * m.n + j];
    } else {
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int k = 0; k < 3; ++k) e.q[a][k] = m.q32[(3 * a + k) * m.n + j];
    }
}

__device__ __forceinline__ void map_point(const Elem32 &e, float s, float t, float w, QPoint<float> &q) {
    if (e.nv == 3) {
        // y - c = (s - 1/3) a + (t - 1/3) b
        float ss = s - (1.0f / 3.0f), tt = t - (1.0f / 3.0f);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            q.d[k] = e.D[k] + ss * e.a[k] + tt * e.b[k];
            q.ny[k] = e.n[k];
        }
        q.wj = w * e.J;
        q.sh[0] = s; q.sh[1] = t; q.sh[2] = 1.0f - s - t; q.sh[3] = 0.0f;
    } else {
        float s1 = 0.25f * (s + 1.0f), s2 = 0.25f * (s - 1.0f), t1 = t + 1.0f, t2 = t - 1.0f;
        float sh[4] = {s1 * t1, -s2 * t1, s2 * t2, -s1 * t2};
        float ds[4], dt[4];
        ds[0] = 0.25f * (t + 1.0f); ds[2] = 0.25f * (t - 1.0f); ds[1] = -ds[0]; ds[3] = -ds[2];
        dt[0] = 0.25f * (s + 1.0f); dt[2] = 0.25f * (s - 1.0f); dt[1] = -dt[2]; dt[3] = -dt[0];
        float dxs[3], dxt[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            float off = 0.f;
            dxs[k] = 0.f; dxt[k] = 0.f;
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                off += sh[a] * e.q[a][k];
                dxs[k] += ds[a] * e.q[a][k];
                dxt[k] += dt[a] * e.q[a][k];
            }
            q.d[k] = e.D[k] + off;
        }
        float nx = dxs[1] * dxt[2] - dxt[1] * dxs[2];
        float ny = dxs[2] * dxt[0] - dxt[2] * dxs[0];
        float nz = dxs[0] * dxt[1] - dxt[0] * dxs[1];
        float len = sqrtf(nx * nx + ny * ny + nz * nz);
        float il = 1.0f / len;
        q.ny[0] = nx * il; q.ny[1] = ny * il; q.ny[2] = nz * il;
        q.wj = w * len;
#pragma unroll
        for (int a = 0; a < 4; ++a) q.sh[a] = sh[a];
    }
    const float r2 = q.d[0] * q.d[0] + q.d[1] * q.d[1] + q.d[2] * q.d[2];
    q.ir = rsqrt_approx(r2);
    q.r = r2 * q.ir;
}

// Kernel values of one quadrature point for a collocation point with normal
// nx (NC_RegularIntegration, NC_EquationSystem.cpp:1691-1717):
//   G  = w e^{i wr r}/(4 pi r),  H = G (-1/r + i wr) (r^.ny),
//   HT = G (-1/r + i wr) (-r^.nx),
//   E  = G [(3/r^2 - k^2) rq + nx.ny/r^2 - i wr/r (3 rq + nx.ny)],
// rq = (r^.ny)(-r^.nx).
template <typename T> struct KVals { cplx<T> G, H, HT, E; };

template <typename T>
__device__ __forceinline__ KVals<T> kernel_values(const QPoint<T> &q, const T nx[3], T k, T wr) {
    const T r = q.r, ir = q.ir;
    T s, c;
    sincos_t(wr * r, &s, &c);
    T amp = q.wj * T(1.0 / kPI4) * ir;
    cplx<T> zg = {c * amp, s * amp};
    cplx<T> z1 = {-ir, wr};
    cplx<T> zh = zg * z1;
    T re1 = (q.d[0] * q.ny[0] + q.d[1] * q.ny[1] + q.d[2] * q.ny[2]) * ir;
    T re2 = -(q.d[0] * nx[0] + q.d[1] * nx[1] + q.d[2] * nx[2]) * ir;
    T rq = re1 * re2;
    T nn = nx[0] * q.ny[0] + nx[1] * q.ny[1] + nx[2] * q.ny[2];
    T ir2 = ir * ir;
    cplx<T> ze1 = {(T(3) * ir2 - k * k) * rq + nn * ir2, -wr * ir * (T(3) * rq + nn)};
    KVals<T> v;
    v.G = zg;
    v.H = zh * re1;
    v.HT = zh * re2;
    v.E = zg * ze1;
    return v;
}

// Physics constants of one frequency.
template <typename T> struct Phys {
    T k, wr;      // wave number, time factor * k
    T tao;        // +1 exterior, -1 interior
    T beta_im;    // Burton-Miller coupling beta = i * beta_im (gamma = 1)
};

// Combine G, H, HT, E of a column into the matrix entry
// (NC_AssembleTBEM, NC_EquationSystem.cpp:165-207).
template <typename T>
__device__ __forceinline__ cplx<T> combine_entry(const KVals<T> &v, int bc, cplx<T> adm, const Phys<T> &P) {
    cplx<T> beta = {T(0), P.beta_im};
    if (bc == 1) {
        // pressure prescribed: -G gamma tao - HT beta
        return v.G * (-P.tao) - v.HT * beta;
    }
    cplx<T> z = v.H * P.tao + v.E * beta;
    if (bc == 2) z += (v.G + v.HT * (beta * P.tao)) * adm;
    return z;
}

}  // namespace bem
