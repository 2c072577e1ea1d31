// bem_kernels.cu - assembly, right-hand side and field-projection kernels.
//
// Every launch covers a batch of systems ((mesh, frequency) instances) whose
// table travels in kernel parameter space (__grid_constant__); a single solve
// is a batch of one.
//
// Regular pairs (k_far): a persistent grid pulls tiles of 32 rows x 32
// columns from a work queue that spans all systems of the batch; in a tile,
// each of 8 warps owns 4 rows and each lane one column, so the column
// element's tables are loaded once per lane and reused for 4 rows, and the
// entries go out as coalesced row segments.  Pairs that NumCalc subdivides
// and the self pairs are skipped there and integrated by k_near: warps pull
// entries of the per-mesh near lists from a second queue and integrate them
// cooperatively (warp_subdivide / warp_singular).
#include <algorithm>
#include <memory>
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
    m.q32 = v.q32; m.isqa32 = v.isqa32; m.n32 = v.n32; m.row4 = v.row4;
    m.sym = v.sym;
    return m;
}

// Largest b with off[b] <= item (off ascending, off[0] = 0, item < off[B]).
__device__ __forceinline__ int find_sys(const int *off, int B, int item) {
    int lo = 0, hi = B - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (off[mid] <= item) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Persistent-grid exit: the last block to leave resets the queue counters
// (ctr[0] = items handed out, ctr[1] = blocks finished) for the next launch.
__device__ __forceinline__ void queue_exit(unsigned *ctr) {
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        __threadfence();
        if (atomicAdd(ctr + 1, 1u) == gridDim.x - 1) {
            ctr[0] = 0u;
            ctr[1] = 0u;
            __threadfence();
        }
    }
}

__device__ __forceinline__ cplx<double> ld_c(const double *p, int idx) {
    double2 v = reinterpret_cast<const double2 *>(p)[idx];
    return {v.x, v.y};
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

// Fused float evaluation of a regular pair's matrix entry.  The entry is
// linear in the kernel values, so each quadrature point contributes
// G * F with F built from the point's geometry and the column's boundary
// condition (NC_AssembleTBEM, NC_EquationSystem.cpp:165-207):
//   velocity:        H tau + E beta            -> F = tau z1 re1 + i b ze1
//   + admittance:    ... + (G + HT beta tau) Y -> F += Y (1 + i b tau z1 re2)
//   pressure:        -G tau - HT beta          -> F = -tau - i b z1 re2
// with z1 = -1/r + i wr, re1 = r^.n_y, re2 = -r^.n_x,
// ze1 = (3/r^2 - k^2) rq + n_x.n_y/r^2 - i wr/r (3 rq + n_x.n_y), rq = re1 re2,
// beta = i b.  One complex accumulator per entry instead of four.
struct FusedCol {
    int bc;
    float yr, yi;          // admittance (bc 2)
    float tau, b, k2, wr;  // tau, beta / i, k^2, time factor * k
};

__device__ __forceinline__ void fused_point(const FusedCol &c, float dny, float dnx, float nn, float r2, float w,
                                            float &acc_re, float &acc_im) {
    const float ir = rsqrt_approx(r2);
    const float r = r2 * ir;
    float sn, cs;
    phase_sincos(c.wr * r, &sn, &cs);
    const float amp = w * (float)(1.0 / kPI4) * ir;
    const float gr = cs * amp, gi = sn * amp;   // G
    const float re1 = dny * ir, re2 = -dnx * ir;
    float fr, fi;
    if (c.bc == 1) {
        // -tau - i b (-ir re2 + i wr re2) = (-tau + b wr re2, b ir re2)
        fr = fmaf(c.b * c.wr, re2, -c.tau);
        fi = c.b * ir * re2;
    } else {
        const float rq = re1 * re2, ir2 = ir * ir;
        const float e_re = fmaf(3.f * ir2 - c.k2, rq, nn * ir2);
        const float e_im = -c.wr * ir * fmaf(3.f, rq, nn);
        // tau z1 re1 + i b ze1
        fr = fmaf(-c.tau * ir, re1, -c.b * e_im);
        fi = fmaf(c.tau * c.wr, re1, c.b * e_re);
        if (c.bc == 2) {
            // Y (1 + i b tau z1 re2) = Y (1 - b tau wr re2, -b tau ir re2)
            const float pr = fmaf(-c.b * c.tau * c.wr, re2, 1.f), pi = -c.b * c.tau * ir * re2;
            fr += c.yr * pr - c.yi * pi;
            fi += c.yr * pi + c.yi * pr;
        }
    }
    acc_re = fmaf(gr, fr, fmaf(-gi, fi, acc_re));
    acc_im = fmaf(gr, fi, fmaf(gi, fr, acc_im));
}

// Points O0 .. O0+NP-1 of the triangle rules, unrolled so that the rule's
// constants are constant-bank operands (the order is uniform across most
// warps: neighbouring columns are neighbouring elements).
template <int NP, int O0>
__device__ __forceinline__ void tri_points(const Elem32 &e, float dny, float dnx0, float anx, float bnx, float nn,
                                           const FusedCol &c, float &ar, float &ai) {
#pragma unroll
    for (int g = 0; g < NP; ++g) {
        const float ss = c_trif[O0 + g][0] - (1.0f / 3.0f), tt = c_trif[O0 + g][1] - (1.0f / 3.0f);
        const float w = c_trif[O0 + g][2] * e.J;
        float d[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) d[k] = fmaf(tt, e.b[k], fmaf(ss, e.a[k], e.D[k]));
        const float r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        fused_point(c, dny, fmaf(tt, bnx, fmaf(ss, anx, dnx0)), nn, r2, w, ar, ai);
    }
}

// Matrix entry of a regular pair in float with a fixed Gauss order.  Flat
// triangles: n_y is constant and d.n_y = D.n_y at every point; d.n_x is
// affine in (s, t).
__device__ __forceinline__ float2 far_entry_f(const Elem32 &e, const float nx[3], int order, const FusedCol &c) {
    float ar = 0.f, ai = 0.f;
    if (e.nv == 3) {
        const float dny = e.D[0] * e.n[0] + e.D[1] * e.n[1] + e.D[2] * e.n[2];
        const float dnx0 = e.D[0] * nx[0] + e.D[1] * nx[1] + e.D[2] * nx[2];
        const float anx = e.a[0] * nx[0] + e.a[1] * nx[1] + e.a[2] * nx[2];
        const float bnx = e.b[0] * nx[0] + e.b[1] * nx[1] + e.b[2] * nx[2];
        const float nn = e.n[0] * nx[0] + e.n[1] * nx[1] + e.n[2] * nx[2];
        if (order <= 2) tri_points<4, 0>(e, dny, dnx0, anx, bnx, nn, c, ar, ai);
        else if (order == 3) tri_points<7, 4>(e, dny, dnx0, anx, bnx, nn, c, ar, ai);
        else tri_points<13, 11>(e, dny, dnx0, anx, bnx, nn, c, ar, ai);
    } else {
        const int np = quad_count(order);
        for (int g = 0; g < np; ++g) {
            const int a = g / order, b = g - a * order;
            QPoint<float> q;
            map_point(e, c_glxf[order][a], c_glxf[order][b], c_glwf[order][a] * c_glwf[order][b], q);
            const float dny = q.d[0] * q.ny[0] + q.d[1] * q.ny[1] + q.d[2] * q.ny[2];
            const float dnx = q.d[0] * nx[0] + q.d[1] * nx[1] + q.d[2] * nx[2];
            const float nn = q.ny[0] * nx[0] + q.ny[1] * nx[1] + q.ny[2] * nx[2];
            const float r2 = q.d[0] * q.d[0] + q.d[1] * q.d[1] + q.d[2] * q.d[2];
            fused_point(c, dny, dnx, nn, r2, q.wj, ar, ai);
        }
    }
    return make_float2(ar, ai);
}

// Order-2 far pair on a flat triangle (the 4-point rule) with the column
// element's data hoisted out of the row loop: point g's squared distance is
// |D|^2 + 2 s_g D.a + 2 t_g D.b + C_g with C_g = |s_g a + t_g b|^2 (at the
// order-2 ratio, |D| > 4 sqrt(area), the terms do not cancel), and the
// kernel terms of fused_point regrouped around u = 1/r.
struct FarCol4 {
    float a[3], b[3], n[3];
    float C[4];    // |s_g a + t_g b|^2
    float J4;      // J / (4 pi)
};

__device__ __forceinline__ void far_col4(const DevMesh &m, int j, FarCol4 &e) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        e.a[k] = m.t32[k * m.n + j];
        e.b[k] = m.t32[(3 + k) * m.n + j];
        e.n[k] = m.t32[(6 + k) * m.n + j];
    }
    const float J = m.t32[9 * m.n + j];
#pragma unroll
    for (int g = 0; g < 4; ++g) {
        float c = 0.f;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float d = fmaf(c_far4[g][1], e.b[k], c_far4[g][0] * e.a[k]);
            c = fmaf(d, d, c);
        }
        e.C[g] = c;
    }
    e.J4 = J * (float)(1.0 / kPI4);
}

// BC: the column's boundary condition (0 velocity, 1 pressure, 2 velocity
// with admittance), fixed per instantiation so the point loop has no branch
template <int BC>
__device__ __forceinline__ float2 far_entry_tri2_bc(const FarCol4 &e, const float D[3], float D2, const float nx[3],
                                                    const FusedCol &c) {
    const float dny = D[0] * e.n[0] + D[1] * e.n[1] + D[2] * e.n[2];
    const float dnx0 = D[0] * nx[0] + D[1] * nx[1] + D[2] * nx[2];
    const float anx = e.a[0] * nx[0] + e.a[1] * nx[1] + e.a[2] * nx[2];
    const float bnx = e.b[0] * nx[0] + e.b[1] * nx[1] + e.b[2] * nx[2];
    const float nn = e.n[0] * nx[0] + e.n[1] * nx[1] + e.n[2] * nx[2];
    const float Da = D[0] * e.a[0] + D[1] * e.a[1] + D[2] * e.a[2];
    const float Db = D[0] * e.b[0] + D[1] * e.b[1] + D[2] * e.b[2];
    const float ct = -c.tau * dny;          // velocity: -tau d.n_y / r^2
    const float cw = c.tau * c.wr * dny;    // velocity: tau wr d.n_y / r
    const float bwr = c.b * c.wr;
    float ar = 0.f, ai = 0.f;
#pragma unroll
    for (int g = 0; g < 4; ++g) {
        const float r2 = fmaf(c_far4[g][2], Da, fmaf(c_far4[g][3], Db, D2 + e.C[g]));
        const float dnx = fmaf(c_far4[g][1], bnx, fmaf(c_far4[g][0], anx, dnx0));
        const float u = rsqrt_approx(r2);
        float sn, cs;
        phase_sincos(c.wr * (r2 * u), &sn, &cs);
        float fr, fi;
        if (BC == 1) {
            // -tau - i b z1 re2, z1 = -1/r + i wr, re2 = -d.n_x / r
            const float du = dnx * u;
            fr = fmaf(-bwr, du, -c.tau);
            fi = -c.b * du * u;
        } else {
            // tau z1 re1 + i b ze1 (re1 = d.n_y / r)
            const float u2 = u * u;
            const float rq = -(dny * dnx) * u2;
            fr = fmaf(bwr * u, fmaf(3.f, rq, nn), ct * u2);
            fi = fmaf(c.b, fmaf(fmaf(3.f, u2, -c.k2), rq, nn * u2), cw * u);
            if (BC == 2) {
                // + Y (1 + i b tau z1 re2)
                const float du = dnx * u, bt = c.b * c.tau;
                const float pr = fmaf(bt * c.wr, du, 1.f), pi = bt * u * du;
                fr += c.yr * pr - c.yi * pi;
                fi += c.yr * pi + c.yi * pr;
            }
        }
        const float amp = c_trif[g][2] * e.J4 * u;
        ar = fmaf(amp, fmaf(cs, fr, -sn * fi), ar);
        ai = fmaf(amp, fmaf(cs, fi, sn * fr), ai);
    }
    return make_float2(ar, ai);
}

__device__ __forceinline__ float2 far_entry_tri2(const FarCol4 &e, const float D[3], float D2, const float nx[3],
                                                 const FusedCol &c) {
    if (c.bc == 0) return far_entry_tri2_bc<0>(e, D, D2, nx, c);
    if (c.bc == 1) return far_entry_tri2_bc<1>(e, D, D2, nx, c);
    return far_entry_tri2_bc<2>(e, D, D2, nx, c);
}

template <typename T>
__device__ __forceinline__ cplx<T> col_adm(const DevFreq &f, int j, int bc) {
    if (bc != 2 || f.adm == nullptr) return {T(0), T(0)};
    cplx<double> a = ld_c(f.adm, j);
    return {(T)a.re, (T)a.im};
}

// ------------------------------------------------------------ symmetry images
// Image tables (DevSym): one thread per (image, element).  The vertices go
// through the reference's sequence of reflections (2 c - x per step, then the
// node swap, NC_ReflectElement, NC_3dFunctions.cpp:357-452), so that each
// image holds the coordinates the reference integrates over; the centre is
// the global point at the local centre, as NC_GenerateSubelements computes
// it for the level-0 test.
__global__ void __launch_bounds__(256) k_image_tables(DevMeshView mv, ImageTables out) {
    const DevMesh m = to_dev(mv);
    const int n = m.n;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)(m.sym.nref - 1) * n) return;
    const int k = (int)(t / n), j = (int)(t - (long long)k * n), kref = k + 1;
    Elem64 e;
    load_elem64(m, j, e);
    double nr[3] = {m.n64[j], m.n64[n + j], m.n64[2 * n + j]};
    for (int step = 1; step <= kref; ++step) {
        const int d = m.sym.rdir[step];
        const double c2 = 2.0 * m.sym.coord[d];
        for (int a = 0; a < e.nv; ++a) e.p[a][d] = __dsub_rn(c2, e.p[a][d]);
        nr[d] = -nr[d];
        for (int q = 0; q < (e.nv == 4 ? 2 : 1); ++q)
            for (int c = 0; c < 3; ++c) {
                const double tmp = e.p[2 * q][c];
                e.p[2 * q][c] = e.p[2 * q + 1][c];
                e.p[2 * q + 1][c] = tmp;
            }
    }
    const size_t nn = (size_t)n, ko = (size_t)k;
    double *v64 = out.v64 + ko * 12 * nn, *c64 = out.c64 + ko * 3 * nn;
    float *chi = out.chi + ko * 3 * nn, *clo = out.clo + ko * 3 * nn;
    float *t32 = out.t32 + ko * 10 * nn, *q32 = out.q32 + ko * 12 * nn;
    for (int a = 0; a < 4; ++a)
        for (int c = 0; c < 3; ++c) v64[(3 * a + c) * nn + j] = a < e.nv ? e.p[a][c] : 0.0;
    // local centre: (1 + 0 + 0) / 3 on triangles, 0 on quadrilaterals
    const double sc = e.nv == 3 ? 1.0 / 3.0 : 0.0;
    double cen[3];
    global_point_exact(e, sc, sc, cen);
    for (int c = 0; c < 3; ++c) {
        c64[c * nn + j] = cen[c];
        const float h = (float)cen[c];
        chi[c * nn + j] = h;
        clo[c * nn + j] = (float)(cen[c] - (double)h);
    }
    if (e.nv == 3) {
        for (int c = 0; c < 3; ++c) {
            t32[c * nn + j] = (float)(e.p[0][c] - e.p[2][c]);
            t32[(3 + c) * nn + j] = (float)(e.p[1][c] - e.p[2][c]);
            t32[(6 + c) * nn + j] = (float)nr[c];
        }
        t32[9 * nn + j] = m.t32[9 * nn + j];
        for (int r = 0; r < 12; ++r) q32[r * nn + j] = 0.f;
    } else {
        for (int r = 0; r < 10; ++r) t32[r * nn + j] = 0.f;
        for (int a = 0; a < 4; ++a)
            for (int c = 0; c < 3; ++c) q32[(3 * a + c) * nn + j] = (float)(e.p[a][c] - cen[c]);
    }
}

// ------------------------------------------------------------ near list
// Pairs (row i, column j) that NumCalc integrates with subdivision (level-0
// ratio distance/sqrt(area) < 1.3, exact FP64 test, for any image of j) plus
// the self pairs.  Depends on the geometry only, so it is built once per
// mesh.  Entries go to list[0, cap) in any order (warp-aggregated atomics);
// *count ends as the number of entries, which may exceed cap (the caller
// then runs again with a larger list).
//
// Bounding spheres of the column blocks (32 consecutive elements, Morton
// order) of every image, and each block's largest sqrt(area): warp per
// (image, block).  Radii are inflated past float rounding, so the block test
// of k_near_list never drops a pair the element test would keep.
__global__ void __launch_bounds__(256) k_block_spheres(DevMeshView mv, float4 *sph, float *bsq) {
    const DevMesh m = to_dev(mv);
    const int lane = threadIdx.x, n = m.n, nb = (n + 31) / 32;
    const int gw = blockIdx.x * 8 + threadIdx.y;
    if (gw >= nb * m.sym.nref) return;
    const int kref = gw / nb, b = gw - kref * nb;
    const DevMesh mk = image_mesh(m, kref);
    const int j = b * 32 + lane, jj = j < n ? j : b * 32;   // idle lanes repeat the block's first element
    float c[3], lo[3], hi[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        c[k] = mk.chi[k * n + jj] + mk.clo[k * n + jj];
        lo[k] = c[k];
        hi[k] = c[k];
        for (int o = 16; o > 0; o >>= 1) {
            lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
            hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
        }
    }
    const float cx = 0.5f * (lo[0] + hi[0]), cy = 0.5f * (lo[1] + hi[1]), cz = 0.5f * (lo[2] + hi[2]);
    float r = sqrtf((c[0] - cx) * (c[0] - cx) + (c[1] - cy) * (c[1] - cy) + (c[2] - cz) * (c[2] - cz));
    float sq = (float)m.sqa64[jj];
    for (int o = 16; o > 0; o >>= 1) {
        r = fmaxf(r, __shfl_xor_sync(0xffffffffu, r, o));
        sq = fmaxf(sq, __shfl_xor_sync(0xffffffffu, sq, o));
    }
    if (lane == 0) {
        const float cmax = fmaxf(fabsf(cx), fmaxf(fabsf(cy), fabsf(cz)));
        sph[gw] = make_float4(cx, cy, cz, r * (1.f + 1e-5f) + 1e-6f * cmax);
        if (kref == 0) bsq[b] = sq * (1.f + 1e-5f);
    }
}

// Near list: warp per row, lanes over 32 column blocks at a time.  A block
// whose sphere (of any image) lies farther from the row's centre than 1.31
// times its largest sqrt(area) holds no pair below the subdivision threshold
// 1.3 (the element test below keeps pairs up to 1.3 (1 + 1e-4) for the exact
// decision); the other blocks get the element test, image by image as the
// reference loops them, with one entry per (row, column) carrying the mask of
// near images (the self pair always).
__global__ void __launch_bounds__(256) k_near_list(DevMeshView mv, const float4 *sph, const float *bsq, int2 *list,
                                                   unsigned long long *count, unsigned long long cap) {
    const DevMesh m = to_dev(mv);
    const int lane = threadIdx.x, n = m.n, nb = (n + 31) / 32, nref = m.sym.nref;
    const int i = blockIdx.x * 8 + threadIdx.y;
    if (i >= n) return;
    const float ci[3] = {m.chi[i] + m.clo[i], m.chi[n + i] + m.clo[n + i], m.chi[2 * n + i] + m.clo[2 * n + i]};
    const float cn = fmaxf(fabsf(ci[0]), fmaxf(fabsf(ci[1]), fabsf(ci[2])));
    for (int cb0 = 0; cb0 < nb; cb0 += 32) {
        const int cb = cb0 + lane;
        bool cand = false;
        if (cb < nb) {
            const float thr = 1.31f * bsq[cb];
            for (int kref = 0; kref < nref; ++kref) {
                const float4 sp = sph[kref * nb + cb];
                const float d0 = ci[0] - sp.x, d1 = ci[1] - sp.y, d2 = ci[2] - sp.z;
                const float slack = 1e-6f * (cn + fmaxf(fabsf(sp.x), fmaxf(fabsf(sp.y), fabsf(sp.z))));
                if (sqrtf(d0 * d0 + d1 * d1 + d2 * d2) - sp.w <= thr + slack) cand = true;
            }
        }
        unsigned cm = __ballot_sync(0xffffffffu, cand);
        while (cm) {
            const int bl = __ffs(cm) - 1;
            cm &= cm - 1;
            const int j = (cb0 + bl) * 32 + lane;
            unsigned imask = 0;
            if (j < n) {
                for (int kref = 0; kref < nref; ++kref) {
                    if (kref == 0 && j == i) { imask |= 1u; continue; }
                    const DevMesh mk = image_mesh(m, kref);
                    const float d0 = (mk.chi[j] - m.chi[i]) + (mk.clo[j] - m.clo[i]);
                    const float d1 = (mk.chi[n + j] - m.chi[n + i]) + (mk.clo[n + j] - m.clo[n + i]);
                    const float d2 = (mk.chi[2 * n + j] - m.chi[2 * n + i]) + (mk.clo[2 * n + j] - m.clo[2 * n + i]);
                    const float rf = sqrtf(d0 * d0 + d1 * d1 + d2 * d2) * m.isqa32[j];
                    if (rf <= 1.3f * (1.0f + 1e-4f)) {
                        const double x[3] = {m.c64[i], m.c64[n + i], m.c64[2 * n + i]};
                        if (ratio0_exact(mk, j, x) < kTolf) imask |= 1u << kref;
                    }
                }
            }
            const bool near = imask != 0;
            const unsigned mask = __ballot_sync(0xffffffffu, near);
            if (!mask) continue;
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(count, (unsigned long long)__popc(mask));
            base = __shfl_sync(0xffffffffu, base, 0);
            const unsigned long long idx = base + __popc(mask & ((1u << lane) - 1u));
            if (near && list && idx < cap) list[idx] = make_int2(i, j | (int)(imask << kNearColBits));
        }
    }
}

// ------------------------------------------------------------ regular pairs
// Regular (not subdivided) pairs: block of 8 warps, every warp 4 rows x 32
// columns, one column per lane.  The column element is loaded once per lane
// and reused for its 4 rows; entries go out as coalesced row segments.  Near
// and self pairs are skipped here and written by k_near.
constexpr int kRowsPerThread = 4;

// Out-of-line parts of the float tile, taken by few pairs: keeping them out
// of the row loop keeps the mesh pointers they read out of its registers.
// Exact (FP64) decision for a pair within the float test's margin of a
// threshold: 0 for a near pair, else the Gauss order.
__device__ __noinline__ int far_order_exact(const DevMeshView *mv, int i, int j) {
    const DevMesh m = to_dev(*mv);
    const int n = m.n;
    const double x64[3] = {m.c64[i], m.c64[n + i], m.c64[2 * n + i]};
    const double rd = ratio0_exact(m, j, x64);
    return rd < kTolf ? 0 : gauss_order(rd);
}
// Entry of a quadrilateral column or of a Gauss order above 2.
__device__ __noinline__ float2 far_entry_general(const DevMeshView *mv, int j, float D0, float D1, float D2,
                                                 float nx0, float nx1, float nx2, int order, FusedCol fc) {
    const DevMesh m = to_dev(*mv);
    Elem32 e;
    const float zero[3] = {0.f, 0.f, 0.f};
    load_elem32(m, j, zero, zero, e);
    e.D[0] = D0; e.D[1] = D1; e.D[2] = D2;
    const float nx[3] = {nx0, nx1, nx2};
    return far_entry_f(e, nx, order, fc);
}

template <typename T>
__device__ __forceinline__ void far_tile(const DevMeshView &mv, const DevFreq &f,
                                         typename Vec2<T>::type *__restrict__ A, size_t lda, int tx, int ty) {
    const DevMesh m = to_dev(mv);
    const int lane = threadIdx.x, n = m.n;
    const int i0 = (ty * 8 + threadIdx.y) * kRowsPerThread;
    const int j = tx * 32 + lane;
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
            // near and self entries: zero here, k_near adds their integrals
            if (i == j) { A[(size_t)i * lda + j] = make_double2(0.0, 0.0); continue; }
            const double x64[3] = {m.c64[i], m.c64[n + i], m.c64[2 * n + i]};
            const double rd = ratio0_exact(m, j, x64);
            if (rd < kTolf) { A[(size_t)i * lda + j] = make_double2(0.0, 0.0); continue; }
            const double nx64[3] = {m.n64[i], m.n64[n + i], m.n64[2 * n + i]};
            KVals<double> v = FarPair<double>::run(e, x64, nx64, gauss_order(rd), f.k, f.wr);
            const cplx<double> val = combine_entry(v, bcj, admj, PT);
            A[(size_t)i * lda + j] = make_double2(val.re, val.im);
        }
    } else {
        const bool tri = m.nvert[j] == 3;
        FarCol4 e4;
        if (tri) far_col4(m, j, e4);
        const float cjh[3] = {m.chi[j], m.chi[n + j], m.chi[2 * n + j]};
        const float cjl[3] = {m.clo[j], m.clo[n + j], m.clo[2 * n + j]};
        const float isq2 = m.isqa32[j] * m.isqa32[j];
        FusedCol fc;
        fc.bc = bcj;
        fc.yr = admj.re;
        fc.yi = admj.im;
        fc.tau = PT.tao;
        fc.b = PT.beta_im;
        fc.k2 = PT.k * PT.k;
        fc.wr = PT.wr;
        #pragma unroll 1
        for (int r = 0; r < kRowsPerThread; ++r) {
            const int i = i0 + r;
            if (i >= n) break;
            if (i == j) { A[(size_t)i * lda + j] = make_float2(0.f, 0.f); continue; }
            // the row's data (the same for the warp's 32 columns)
            const float4 rh = m.row4[3 * (size_t)i], rl = m.row4[3 * (size_t)i + 1], rn = m.row4[3 * (size_t)i + 2];
            const float D[3] = {(cjh[0] - rh.x) + (cjl[0] - rl.x), (cjh[1] - rh.y) + (cjl[1] - rl.y),
                                (cjh[2] - rh.z) + (cjl[2] - rl.z)};
            const float D2 = D[0] * D[0] + D[1] * D[1] + D[2] * D[2];
            const float q2 = D2 * isq2;
            bool near = false;
            int order = 2;
            if (q2 <= c_quad.far2_sq && !classify_fast(sqrtf(q2), near, order)) {
                order = far_order_exact(&mv, i, j);
                near = order == 0;
            }
            if (near) { A[(size_t)i * lda + j] = make_float2(0.f, 0.f); continue; }
            const float nx[3] = {rn.x, rn.y, rn.z};
            if (tri && order <= 2)
                A[(size_t)i * lda + j] = far_entry_tri2(e4, D, D2, nx, fc);
            else
                A[(size_t)i * lda + j] = far_entry_general(&mv, j, D[0], D[1], D[2], nx[0], nx[1], nx[2], order, fc);
        }
    }
}

// The same tile for a mesh with symmetry images: every entry sums the far
// images of its column element (reflection factor applied, NC_AssembleTBEM,
// NC_EquationSystem.cpp:181-206), in image order; near images and the self
// pair are left to k_near, which adds them to the entry.
template <typename T>
__device__ __forceinline__ void far_tile_img(const DevMeshView &mv, const DevFreq &f,
                                             typename Vec2<T>::type *__restrict__ A, size_t lda, int tx, int ty) {
    const DevMesh m = to_dev(mv);
    const int lane = threadIdx.x, n = m.n;
    const int i0 = (ty * 8 + threadIdx.y) * kRowsPerThread;
    const int j = tx * 32 + lane;
    if (i0 >= n || j >= n) return;
    Phys<T> PT;
    if constexpr (std::is_same<T, double>::value) PT = {f.k, f.wr, f.tao, f.beta_im};
    else PT = {f.kf, f.wrf, f.taof, f.beta_imf};
    const int bcj = f.bc_type ? f.bc_type[j] : 0;
    const cplx<T> admj = col_adm<T>(f, j, bcj);
    T acc_re[kRowsPerThread], acc_im[kRowsPerThread];
    for (int r = 0; r < kRowsPerThread; ++r) acc_re[r] = acc_im[r] = T(0);
    for (int kref = 0; kref < m.sym.nref; ++kref) {
        const DevMesh mk = image_mesh(m, kref);
        const T sg = image_negated(m, kref) ? T(-1) : T(1);
        if constexpr (std::is_same<T, double>::value) {
            Elem64 e;
            load_elem64(mk, j, e);
            for (int r = 0; r < kRowsPerThread; ++r) {
                const int i = i0 + r;
                if (i >= n) break;
                if (kref == 0 && i == j) continue;
                const double x64[3] = {m.c64[i], m.c64[n + i], m.c64[2 * n + i]};
                const double rd = ratio0_exact(mk, j, x64);
                if (rd < kTolf) continue;
                const double nx64[3] = {m.n64[i], m.n64[n + i], m.n64[2 * n + i]};
                KVals<double> v = FarPair<double>::run(e, x64, nx64, gauss_order(rd), f.k, f.wr);
                const cplx<double> val = combine_entry(v, bcj, admj, PT);
                acc_re[r] += sg * val.re;
                acc_im[r] += sg * val.im;
            }
        } else {
            Elem32 e;
            const float zero[3] = {0.f, 0.f, 0.f};
            load_elem32(mk, j, zero, zero, e);
            const float cjh[3] = {mk.chi[j], mk.chi[n + j], mk.chi[2 * n + j]};
            const float cjl[3] = {mk.clo[j], mk.clo[n + j], mk.clo[2 * n + j]};
            const float isq2 = m.isqa32[j] * m.isqa32[j];
            FusedCol fc;
            fc.bc = bcj;
            fc.yr = admj.re;
            fc.yi = admj.im;
            fc.tau = PT.tao;
            fc.b = PT.beta_im;
            fc.k2 = PT.k * PT.k;
            fc.wr = PT.wr;
            for (int r = 0; r < kRowsPerThread; ++r) {
                const int i = i0 + r;
                if (i >= n) break;
                if (kref == 0 && i == j) continue;
                for (int k = 0; k < 3; ++k) e.D[k] = (cjh[k] - m.chi[k * n + i]) + (cjl[k] - m.clo[k * n + i]);
                const float q2 = (e.D[0] * e.D[0] + e.D[1] * e.D[1] + e.D[2] * e.D[2]) * isq2;
                bool near = false;
                int order = 2;
                if (q2 <= c_quad.far2_sq && !classify_fast(sqrtf(q2), near, order)) {
                    const double x64[3] = {m.c64[i], m.c64[n + i], m.c64[2 * n + i]};
                    const double rd = ratio0_exact(mk, j, x64);
                    near = rd < kTolf;
                    if (!near) order = gauss_order(rd);
                }
                if (near) continue;
                const float nx[3] = {m.n32[i], m.n32[n + i], m.n32[2 * n + i]};
                const float2 v = far_entry_f(e, nx, order, fc);
                acc_re[r] += sg * v.x;
                acc_im[r] += sg * v.y;
            }
        }
    }
    for (int r = 0; r < kRowsPerThread; ++r) {
        const int i = i0 + r;
        if (i >= n) break;
        typename Vec2<T>::type o;
        o.x = acc_re[r];
        o.y = acc_im[r];
        A[(size_t)i * lda + j] = o;
    }
}

constexpr int kFarPerSm = kFarPerSmMax;   // resident k_far blocks per SM allowed by the launch bounds

// ONE: the batch holds a single system, whose table then stays in constant
// operands instead of registers.  IMG: some mesh of the batch has symmetry
// images (meshes without take the plain tile).
template <typename T, bool ONE, bool IMG>
__global__ void __launch_bounds__(256, kFarPerSm) k_far(const __grid_constant__ AsmBatch tb, unsigned *ctr) {
    __shared__ int item_s;
    const int total = tb.far_off[tb.B];
    while (true) {
        if (threadIdx.x == 0 && threadIdx.y == 0) item_s = (int)atomicAdd(ctr, 1u);
        __syncthreads();
        const int item = item_s;
        __syncthreads();
        if (item >= total) break;
        const int b = ONE ? 0 : find_sys(tb.far_off, tb.B, item);
        const AsmSys &S = tb.sys[ONE ? 0 : b];
        const int local = item - tb.far_off[b];
        const int ntx = (S.m.n + 31) / 32;
        if (IMG && S.m.sym.nref > 1)
            far_tile_img<T>(S.m, S.f, (typename Vec2<T>::type *)S.A, S.lda, local % ntx, local / ntx);
        else
            far_tile<T>(S.m, S.f, (typename Vec2<T>::type *)S.A, S.lda, local % ntx, local / ntx);
    }
    queue_exit(ctr);
}

// ------------------------------------------------------------ near pairs
// One warp per entry of the near list: the self pair by warp_singular (FP64;
// warp_singular_f in FP32 for complex64 systems) plus NumCalc's free term,
// subdivided pairs by warp_subdivide with the
// kernel arithmetic in T; with symmetry planes every image of the entry's
// mask in image order.  The sum is added to the entry k_far wrote (its far
// images, or zero).
template <typename T>
__device__ __forceinline__ void near_pair(const DevMeshView &mv, const DevFreq &f, int2 ij,
                                          typename Vec2<T>::type *__restrict__ A, size_t lda, int *status,
                                          WarpScratch &ws) {
    const DevMesh m = to_dev(mv);
    const int lane = threadIdx.x, n = m.n;
    const int i = ij.x, j = ij.y & kMaxElements;
    const unsigned imask = (unsigned)ij.y >> kNearColBits;
    const double x64[3] = {m.c64[i], m.c64[n + i], m.c64[2 * n + i]};
    const double nx64[3] = {m.n64[i], m.n64[n + i], m.n64[2 * n + i]};
    Phys<double> P{f.k, f.wr, f.tao, f.beta_im};
    Phys<T> PT{(T)f.k, (T)f.wr, (T)f.tao, (T)f.beta_im};
    const int bcj = f.bc_type ? f.bc_type[j] : 0;
    cplx<T> sum = {T(0), T(0)};
    int err = kDevOk;
    for (int kref = 0; kref < 8; ++kref) {
        if (!((imask >> kref) & 1u)) continue;
        const DevMesh mk = image_mesh(m, kref);
        Elem64 e;
        load_elem64(mk, j, e);
        cplx<T> entry;
        if (kref == 0 && i == j) {
            KVals<double> sv;
            if constexpr (std::is_same<T, float>::value) {
                // FP32 rule on the vertices relative to the collocation point
                float pl[4][3];
#pragma unroll
                for (int a = 0; a < 4; ++a)
#pragma unroll
                    for (int k = 0; k < 3; ++k) pl[a][k] = a < e.nv ? (float)(e.p[a][k] - x64[k]) : 0.f;
                const float nxf[3] = {(float)nx64[0], (float)nx64[1], (float)nx64[2]};
                const KVals<float> vf = warp_singular_f(e.nv, pl, nxf, f.kf, f.wrf);
                sv.G = {vf.G.re, vf.G.im};
                sv.H = {vf.H.re, vf.H.im};
                sv.HT = {vf.HT.re, vf.HT.im};
                sv.E = {vf.E.re, vf.E.im};
            } else {
                sv = warp_singular(e, x64, nx64, P, 0, nullptr).v;
            }
            cplx<double> a = combine_entry(sv, bcj, col_adm<double>(f, j, bcj), P);
            // free term, NC_EquationSystem.cpp:220-231
            const cplx<double> beta = {0.0, P.beta_im};
            if (bcj == 1) a += beta * (-(0.5 * P.tao));
            else a += (col_adm<double>(f, j, bcj) * beta - cplx<double>{1.0, 0.0}) * 0.5;
            entry = {(T)a.re, (T)a.im};
        } else if constexpr (std::is_same<T, double>::value) {
            // float tables only for the subdivision's fast decisions
            const float xhi[3] = {m.chi[i], m.chi[n + i], m.chi[2 * n + i]};
            const float xlo[3] = {m.clo[i], m.clo[n + i], m.clo[2 * n + i]};
            Elem32 ef;
            load_elem32(mk, j, xhi, xlo, ef);
            AsmSink<double> sink;
            sink.e = &e; sink.x = x64; sink.nx = nx64; sink.k = f.k; sink.wr = f.wr;
            sink.init();
            const int rc = warp_subdivide(e, m.area64[j], x64, ws, sink, &ef, m.isqa32[j]);
            if (rc != kDevOk) err = rc;
            KVals<double> v = sink.reduce();
            entry = combine_entry(v, bcj, col_adm<double>(f, j, bcj), PT);
        } else {
            const float xhi[3] = {m.chi[i], m.chi[n + i], m.chi[2 * n + i]};
            const float xlo[3] = {m.clo[i], m.clo[n + i], m.clo[2 * n + i]};
            const float nx32[3] = {(float)nx64[0], (float)nx64[1], (float)nx64[2]};
            Elem32 e32;
            load_elem32(mk, j, xhi, xlo, e32);
            AsmSink<float> sink;
            sink.e = &e32; sink.nx = nx32; sink.k = PT.k; sink.wr = PT.wr;
            sink.init();
            const int rc = warp_subdivide(e, m.area64[j], x64, ws, sink, &e32, m.isqa32[j]);
            if (rc != kDevOk) err = rc;
            KVals<float> v = sink.reduce();
            entry = combine_entry(v, bcj, col_adm<float>(f, j, bcj), PT);
        }
        if (image_negated(m, kref)) entry = entry * T(-1);
        sum += entry;
    }
    if (lane == 0) {
        typename Vec2<T>::type o = A[(size_t)i * lda + j];
        o.x += sum.re;
        o.y += sum.im;
        A[(size_t)i * lda + j] = o;
        if (err != kDevOk) atomicMax(status, err);
    }
}

template <typename T>
__global__ void __launch_bounds__(256, 2) k_near(const __grid_constant__ AsmBatch tb, unsigned *ctr) {
    __shared__ WarpScratch ws_all[8];
    WarpScratch &ws = ws_all[threadIdx.y];
    const int total = tb.near_off[tb.B];
    while (true) {
        int item = 0;
        if (threadIdx.x == 0) item = (int)atomicAdd(ctr, 1u);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= total) break;
        const int b = find_sys(tb.near_off, tb.B, item);
        const AsmSys &S = tb.sys[b];
        const int2 ij = S.near[item - tb.near_off[b]];
        near_pair<T>(S.m, S.f, ij, (typename Vec2<T>::type *)S.A, S.lda, S.status, ws);
        __syncwarp();
    }
    queue_exit(ctr);
}

// Images of the incident waves in the symmetry planes: step kref reflects a
// plane-wave direction (negates one component) or a point source (2 c - x)
// across the plane normal to axis rdir[kref]; the reflection factor of image
// kref is the element images' (NC_ReflectPointVector, NC_3dFunctions.cpp:181-242).
__device__ __forceinline__ void reflect_source(const DevSym &sy, int kref, double v[3], bool point) {
    const int d = sy.rdir[kref];
    if (point) v[d] = __dsub_rn(2.0 * sy.coord[d], v[d]);
    else v[d] = -v[d];
}

// Plane waves take their phase at x minus the positions of the planes
// present (NC_EquationSystem.cpp:1743-1748, NC_PostProcessing.cpp:794-799).
__device__ __forceinline__ void plane_wave_origin(const DevSym &sy, const double x[3], double xs[3]) {
    for (int k = 0; k < 3; ++k) xs[k] = ((sy.axes >> k) & 1u) ? x[k] - sy.coord[k] : x[k];
}

// Incident waves at a collocation point (NC_IncidentWaveRHS,
// NC_EquationSystem.cpp:1731-1812), with their symmetry-plane images.
__device__ cplx<double> incident_rhs(const DevSym &sy, const DevFreq &f, const double x[3], const double nx[3]) {
    cplx<double> zrc = {0.0, 0.0};
    const cplx<double> bt = {0.0, f.beta_im * f.tao};
    double xs[3];
    plane_wave_origin(sy, x, xs);
    for (int s = 0; s < f.n_plane; ++s) {
        double d[3] = {f.pw_dir[3 * s], f.pw_dir[3 * s + 1], f.pw_dir[3 * s + 2]};
        const cplx<double> amp = ld_c(f.pw_amp, s);
        for (int kref = 0; kref < sy.nref; ++kref) {
            if (kref > 0) reflect_source(sy, kref, d, false);
            const double rf = ((sy.rneg >> kref) & 1u) ? -1.0 : 1.0;
            const double ph = (d[0] * xs[0] + d[1] * xs[1] + d[2] * xs[2]) * f.wr;
            double sn, cs;
            sincos(ph, &sn, &cs);
            const cplx<double> zg = cplx<double>{cs * rf, sn * rf} * amp;
            const double re1 = f.wr * (d[0] * nx[0] + d[1] * nx[1] + d[2] * nx[2]);
            const cplx<double> zv = {-zg.im * re1, zg.re * re1};
            zrc -= zg + zv * bt;
        }
    }
    for (int s = 0; s < f.n_point; ++s) {
        double p[3] = {f.ps_xyz[3 * s], f.ps_xyz[3 * s + 1], f.ps_xyz[3 * s + 2]};
        const cplx<double> amp = ld_c(f.ps_amp, s);
        for (int kref = 0; kref < sy.nref; ++kref) {
            if (kref > 0) reflect_source(sy, kref, p, true);
            const double rf = ((sy.rneg >> kref) & 1u) ? -1.0 : 1.0;
            double d[3] = {x[0] - p[0], x[1] - p[1], x[2] - p[2]};
            const double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            d[0] /= r; d[1] /= r; d[2] /= r;
            double sn, cs;
            sincos(f.wr * r, &sn, &cs);
            const double re2 = rf / kPI4 / r;
            const cplx<double> zg = cplx<double>{cs * re2, sn * re2} * amp;
            const double re1 = d[0] * nx[0] + d[1] * nx[1] + d[2] * nx[2];
            const cplx<double> zv = cplx<double>{-re1 / r, f.wr * re1} * zg;
            zrc -= zg + zv * bt;
        }
    }
    return zrc;
}

// Right-hand side, one warp per row (FP64): free term of the prescribed value
// (NC_EquationSystem.cpp:233-244), incident waves, and the columns whose
// prescribed values are nonzero (Zrsintel[4], NC_EquationSystem.cpp:188-198),
// each with all its images: nodal values in the image's node order, velocity
// values negated with the reflection factor, no factor on the term itself
// (NC_ReflectElement, NC_3dFunctions.cpp:410-415; NC_AssembleTBEM).
__global__ void __launch_bounds__(256) k_rhs(const __grid_constant__ AsmBatch tb) {
    __shared__ WarpScratch ws_all[8];
    const int sb = find_sys(tb.rhs_off, tb.B, blockIdx.x);
    const AsmSys &S = tb.sys[sb];
    const DevMesh m = to_dev(S.m);
    const DevFreq &f = S.f;
    double2 *b = (double2 *)S.b;
    int *status = S.status;
    const int lane = threadIdx.x, w = threadIdx.y;
    const int n = m.n;
    const int i = (blockIdx.x - tb.rhs_off[sb]) * 8 + w;
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
        if (f.n_plane + f.n_point > 0) z0 += incident_rhs(m.sym, f, x, nx);
    }
    int err = kDevOk;
    for (int c = 0; c < f.n_bc_cols; ++c) {
        const int jc = f.bc_cols[c];
        const int bcj = f.bc_type ? f.bc_type[jc] : 0;
        const int nvj = m.nvert[jc];
        for (int kref = 0; kref < m.sym.nref; ++kref) {
            const DevMesh mk = image_mesh(m, kref);
            Elem64 e;
            load_elem64(mk, jc, e);
            const double vs = (bcj != 1 && image_negated(m, kref)) ? -1.0 : 1.0;
            cplx<double> bc[4];
            for (int a = 0; a < 4; ++a)
                bc[a] = a < nvj ? ld_c(f.bc_val, image_node(a, kref, nvj) * n + jc) * vs : cplx<double>{0.0, 0.0};
            cplx<double> contrib;
            if (kref == 0 && jc == i) {
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
    }
    if (lane == 0) {
        b[i] = make_double2(z0.re, z0.im);
        if (err != kDevOk) atomicMax(status, err);
    }
}

// Element potentials and nodal normal velocities after the solve
// (NC_WriteResultsObjectMesh, NC_PostProcessing.cpp:389-410).
__global__ void __launch_bounds__(256) k_fields(const __grid_constant__ ProjBatch tb) {
    const int sb = find_sys(tb.fld_off, tb.B, blockIdx.x);
    const ProjSys &S = tb.sys[sb];
    const DevMeshView &mv = S.m;
    const DevFreq &f = S.f;
    const double2 *x = (const double2 *)S.x;
    double2 *phi = (double2 *)S.phi, *vel = (double2 *)S.vel;
    int *ivi = S.ivi;
    const int j = (blockIdx.x - tb.fld_off[sb]) * blockDim.x + threadIdx.x;
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
    float2 *phi32 = (float2 *)S.phi32, *vel32 = (float2 *)S.vel32;
    phi32[j] = make_float2((float)p.re, (float)p.im);
    for (int a = 0; a < 4; ++a) vel32[a * n + j] = make_float2((float)v[a].re, (float)v[a].im);
    ivi[j] = any;
}

// Far-pair projection of a flat triangle without velocity terms, fused
// (NC_IntegrationTBEM, NC_PostProcessing.cpp:1217-1322, with phi factored out
// of the quadrature sum): per point Gw = w J e^{i wr r}/(4 pi r), Gi =
// Gw (-1/r + i wr), r^.n_y = (D.n_y)/r (constant numerator on a flat
// element);
//   P  += Gi (r^.n_y)
//   U  += Gw [(r^.n_y)(k^2 - 3/r^2) + i 3 wr (r^.n_y)/r] / r * (y - x)
//   T  -= Gi / r
// and the element adds phi P to the potential and phi (U + T n_y) to the
// gradient.
template <int NP, int O0>
__device__ __forceinline__ void proj_tri_points(const Elem32 &e, float dny, float k2, float wr, float2 &P,
                                                float2 (&U)[3], float2 &T) {
#pragma unroll
    for (int g = 0; g < NP; ++g) {
        const float ss = c_trif[O0 + g][0] - (1.0f / 3.0f), tt = c_trif[O0 + g][1] - (1.0f / 3.0f);
        const float wj = c_trif[O0 + g][2] * e.J * (float)(1.0 / kPI4);
        float d[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) d[k] = fmaf(tt, e.b[k], fmaf(ss, e.a[k], e.D[k]));
        const float r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        const float ir = rsqrt_approx(r2), r = r2 * ir;
        float sn, cs;
        phase_sincos(wr * r, &sn, &cs);
        const float amp = wj * ir;
        const float gr = cs * amp, gi = sn * amp;                              // Gw
        const float hr = fmaf(-gr, ir, -gi * wr), hi = fmaf(gr, wr, -gi * ir);   // Gi
        const float dn = dny * ir;                                           // r^.n_y
        P.x = fmaf(hr, dn, P.x);
        P.y = fmaf(hi, dn, P.y);
        const float ir2 = ir * ir;
        const float f1r = dn * (k2 - 3.0f * ir2), f1i = 3.0f * wr * dn * ir;
        const float ur = (gr * f1r - gi * f1i) * ir, ui = (gr * f1i + gi * f1r) * ir;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            U[k].x = fmaf(ur, d[k], U[k].x);
            U[k].y = fmaf(ui, d[k], U[k].y);
        }
        T.x = fmaf(-hr, ir, T.x);
        T.y = fmaf(-hi, ir, T.y);
    }
}

// Element data of image kref for the projection: potential and nodal
// velocities times the reflection factor, velocities in the image's node
// order (NC_ContributionTBEM, NC_PostProcessing.cpp:925-940).
template <typename T>
__device__ __forceinline__ void proj_elem_data(const double2 *phi, const double2 *vel, const float2 *phi32,
                                               const float2 *vel32, int n, int j, int nv, bool iv, int kref,
                                               bool neg, cplx<T> &ph, cplx<T> vl[4]) {
    const T sg = neg ? T(-1) : T(1);
    if constexpr (std::is_same<T, double>::value) {
        ph = cplx<T>{phi[j].x, phi[j].y} * sg;
        for (int a = 0; a < 4; ++a) {
            const int src = image_node(a, kref, nv);
            vl[a] = (iv && a < nv) ? cplx<T>{vel[src * n + j].x, vel[src * n + j].y} * sg : cplx<T>{0, 0};
        }
    } else {
        const float2 p2 = phi32[j];
        ph = cplx<T>{p2.x, p2.y} * sg;
        for (int a = 0; a < 4; ++a) {
            const float2 v2 = (iv && a < nv) ? vel32[image_node(a, kref, nv) * n + j] : make_float2(0.f, 0.f);
            vl[a] = cplx<T>{v2.x, v2.y} * sg;
        }
    }
}

// Potential and gradient of point p from the element sums (FP64): the tau
// factor, then the incident field with its images (NC_ContributionIncidentWaves,
// NC_PostProcessing.cpp:776-866).
__device__ void project_finish(const DevMesh &m, const DevFreq &f, const double x64[3], int p, cplx<double> sp,
                               cplx<double> sg[3], double2 *pot, double2 *grad) {
    if (f.tao != 1.0) {
        sp = sp * f.tao;
        for (int kk = 0; kk < 3; ++kk) sg[kk] = sg[kk] * f.tao;
    }
    if (f.n_plane || f.n_point) {
        const DevSym &sy = m.sym;
        double xs[3];
        plane_wave_origin(sy, x64, xs);
        for (int s = 0; s < f.n_plane; ++s) {
            double d[3] = {f.pw_dir[3 * s], f.pw_dir[3 * s + 1], f.pw_dir[3 * s + 2]};
            const cplx<double> amp = ld_c(f.pw_amp, s);
            for (int kref = 0; kref < sy.nref; ++kref) {
                if (kref > 0) reflect_source(sy, kref, d, false);
                const double rf = ((sy.rneg >> kref) & 1u) ? -1.0 : 1.0;
                double sn, cs;
                sincos((d[0] * xs[0] + d[1] * xs[1] + d[2] * xs[2]) * f.wr, &sn, &cs);
                const cplx<double> zg = cplx<double>{cs * rf, sn * rf} * amp;
                sp += zg;
                const cplx<double> zv = {-zg.im * f.wr, zg.re * f.wr};
                for (int kk = 0; kk < 3; ++kk) sg[kk] += zv * d[kk];
            }
        }
        for (int s = 0; s < f.n_point; ++s) {
            double q[3] = {f.ps_xyz[3 * s], f.ps_xyz[3 * s + 1], f.ps_xyz[3 * s + 2]};
            const cplx<double> amp = ld_c(f.ps_amp, s);
            for (int kref = 0; kref < sy.nref; ++kref) {
                if (kref > 0) reflect_source(sy, kref, q, true);
                const double rf = ((sy.rneg >> kref) & 1u) ? -1.0 : 1.0;
                double d[3] = {x64[0] - q[0], x64[1] - q[1], x64[2] - q[2]};
                const double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                d[0] /= r; d[1] /= r; d[2] /= r;
                double sn, cs;
                sincos(f.wr * r, &sn, &cs);
                const double re2 = rf / kPI4 / r;
                const cplx<double> zg = cplx<double>{cs * re2, sn * re2} * amp;
                sp += zg;
                const cplx<double> zv = cplx<double>{-1.0 / r, f.wr} * zg;
                for (int kk = 0; kk < 3; ++kk) sg[kk] += zv * d[kk];
            }
        }
    }
    pot[p] = make_double2(sp.re, sp.im);
    if (grad)
        for (int kk = 0; kk < 3; ++kk) grad[3 * p + kk] = make_double2(sg[kk].re, sg[kk].im);
}

// Field projection, one warp per point: lanes sweep the elements (and their
// symmetry images) 32 at a time; regular pairs in the lane, subdivided pairs
// by the whole warp.
template <typename T>
__global__ void __launch_bounds__(256, 2) k_project(const __grid_constant__ ProjBatch tb) {
    __shared__ WarpScratch ws_all[8];
    const int sb = find_sys(tb.pt_off, tb.B, blockIdx.x);
    const ProjSys &S = tb.sys[sb];
    const DevMesh m = to_dev(S.m);
    const DevFreq &f = S.f;
    const double2 *phi = (const double2 *)S.phi, *vel = (const double2 *)S.vel;
    const float2 *phi32 = (const float2 *)S.phi32, *vel32 = (const float2 *)S.vel32;
    const int *ivi = S.ivi;
    const int npts = S.npts;
    const double *pts = S.pts;
    double2 *pot = (double2 *)S.pot, *grad = (double2 *)S.grad;
    int *status = S.status;
    const int lane = threadIdx.x, w = threadIdx.y;
    const int n = m.n;
    const int p = (blockIdx.x - tb.pt_off[sb]) * 8 + w;
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
    for (int kref = 0; kref < m.sym.nref; ++kref) {
        const DevMesh mk = image_mesh(m, kref);
        const bool neg = image_negated(m, kref);
        for (int base = 0; base < n; base += 32) {
            const int j = base + lane;
            const bool valid = j < n;
            bool near = false;
            int order = 2;
            if (valid) {
                // element data in T (float copies for the float path: no FP64 conversions)
                const bool iv = ivi[j] != 0;
                const int nv = m.nvert[j];
                cplx<T> ph, vl[4];
                proj_elem_data<T>(phi, vel, phi32, vel32, n, j, nv, iv, kref, neg, ph, vl);
                if constexpr (std::is_same<T, double>::value) {
                    const double rd = ratio0_exact(mk, j, x64);
                    near = rd < kTolf;
                    if (!near) {
                        order = gauss_order(rd);
                        Elem64 e;
                        load_elem64(mk, j, e);
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
                    load_elem32(mk, j, xhi, xlo, e);
                    const float q2 = (e.D[0] * e.D[0] + e.D[1] * e.D[1] + e.D[2] * e.D[2]) * (m.isqa32[j] * m.isqa32[j]);
                    if (q2 <= c_quad.far2_sq && !classify_fast(sqrtf(q2), near, order)) {
                        const double rd = ratio0_exact(mk, j, x64);
                        near = rd < kTolf;
                        if (!near) order = gauss_order(rd);
                    }
                    if (!near && e.nv == 3 && !iv) {
                        // fused flat-triangle path (no velocity terms)
                        float2 P = make_float2(0.f, 0.f), U[3], Tn = make_float2(0.f, 0.f);
                        U[0] = U[1] = U[2] = make_float2(0.f, 0.f);
                        const float dny = e.D[0] * e.n[0] + e.D[1] * e.n[1] + e.D[2] * e.n[2];
                        const float k2 = (float)k * (float)k;
                        if (order <= 2) proj_tri_points<4, 0>(e, dny, k2, (float)wr, P, U, Tn);
                        else if (order == 3) proj_tri_points<7, 4>(e, dny, k2, (float)wr, P, U, Tn);
                        else proj_tri_points<13, 11>(e, dny, k2, (float)wr, P, U, Tn);
                        const cplx<float> pp = ph * cplx<float>{P.x, P.y};
                        acc.p.re += pp.re;
                        acc.p.im += pp.im;
#pragma unroll
                        for (int kk = 0; kk < 3; ++kk) {
                            const cplx<float> gg = ph * cplx<float>{fmaf(Tn.x, e.n[kk], U[kk].x), fmaf(Tn.y, e.n[kk], U[kk].y)};
                            acc.g[kk].re += gg.re;
                            acc.g[kk].im += gg.im;
                        }
                    } else if (!near) {
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
                load_elem64(mk, jl, e);
                const bool iv = ivi[jl] != 0;
                cplx<T> ph, vl[4];
                proj_elem_data<T>(phi, vel, phi32, vel32, n, jl, e.nv, true, kref, neg, ph, vl);
                ProjAcc<T> r;
                int rc;
                if constexpr (std::is_same<T, double>::value) {
                    ProjSink<double> sink;
                    sink.e = &e; sink.x = x64; sink.phi = ph; sink.vel = vl; sink.ivi = iv; sink.k = k; sink.wr = wr;
                    sink.init();
                    rc = warp_subdivide(e, m.area64[jl], x64, ws, sink);
                    r = sink.reduce();
                } else {
                    Elem32 e32;   // float tables: the arithmetic and the fast decisions
                    load_elem32(mk, jl, xhi, xlo, e32);
                    ProjSink<float> sink;
                    sink.e = &e32; sink.phi = ph; sink.vel = vl; sink.ivi = iv; sink.k = k; sink.wr = wr;
                    sink.init();
                    rc = warp_subdivide(e, m.area64[jl], x64, ws, sink, &e32, m.isqa32[jl]);
                    r = sink.reduce();
                }
                if (rc != kDevOk) err = rc;
                if (lane == 0) {
                    acc.p += r.p;
                    for (int kk = 0; kk < 3; ++kk) acc.g[kk] += r.g[kk];
                }
            }
        }
    }
    // FP64 cross-lane reduction
    cplx<double> sp = warp_sum(cplx<double>{(double)acc.p.re, (double)acc.p.im});
    cplx<double> sg[3];
    for (int kk = 0; kk < 3; ++kk) sg[kk] = warp_sum(cplx<double>{(double)acc.g[kk].re, (double)acc.g[kk].im});
    if (lane == 0) {
        project_finish(m, f, x64, p, sp, sg, pot, grad);
        if (err != kDevOk) atomicMax(status, err);
    }
}

// Float projection with the roles of lanes and elements exchanged: a warp
// takes 32 evaluation points (one per lane) and a slice of the elements,
// and sweeps the slice one element at a time, so every element's data is a
// warp-uniform load shared by 32 points instead of 32 loads of different
// elements.  Partial sums go to ProjSys::part per (slice, point);
// k_project_sum adds the slices in slice order (FP64) and finishes the
// point.  Pair arithmetic as in k_project<float>: the fused flat-triangle
// rule, the general rule, and the warp-wide subdivision for near pairs, here
// one near lane at a time.
constexpr int kProjSlice = 256;   // elements per slice (fewer slices if the scratch is short)

__global__ void __launch_bounds__(256, 2) k_project_pts(const __grid_constant__ ProjBatch tb) {
    __shared__ WarpScratch ws_all[8];
    const int sb = find_sys(tb.lp_off, tb.B, blockIdx.x);
    const ProjSys &S = tb.sys[sb];
    const DevMesh m = to_dev(S.m);
    const DevFreq &f = S.f;
    const int lane = threadIdx.x, w = threadIdx.y, n = m.n, npts = S.npts;
    const int G = (npts + 31) >> 5, nsl = S.nslice;
    const int item = (blockIdx.x - tb.lp_off[sb]) * 8 + w;
    if (item >= G * nsl) return;
    const int g = item % G, sl = item / G;
    const int per = (n + nsl - 1) / nsl;
    const int j0 = sl * per, j1 = min(n, j0 + per);
    const int p = g * 32 + lane;
    const bool pv = p < npts;
    const int pp = pv ? p : g * 32;   // idle lanes shadow the group's first point
    WarpScratch &ws = ws_all[w];
    // The point as float hi/lo pair and the wave numbers in float, made opaque
    // to the compiler: under register pressure it otherwise recomputes them
    // from the FP64 values at every pair, and GB300 issues those conversions
    // (and the FP64 subtraction) on its narrow FP64 pipe.
    float xhi[3], xlo[3];
    for (int c = 0; c < 3; ++c) {
        const double xv = S.pts[3 * pp + c];
        xhi[c] = (float)xv;
        xlo[c] = (float)(xv - (double)xhi[c]);
        asm volatile("" : "+f"(xhi[c]), "+f"(xlo[c]));
    }
    const double2 *phi = (const double2 *)S.phi, *vel = (const double2 *)S.vel;
    const float2 *phi32 = (const float2 *)S.phi32, *vel32 = (const float2 *)S.vel32;
    ProjAcc<float> acc;
    acc.p = acc.g[0] = acc.g[1] = acc.g[2] = cmk(0.f, 0.f);
    float k = (float)f.k, wr = (float)f.wr;
    asm volatile("" : "+f"(k), "+f"(wr));
    const float k2 = k * k;
    int err = kDevOk;
    for (int kref = 0; kref < m.sym.nref; ++kref) {
        const DevMesh mk = image_mesh(m, kref);
        const bool neg = image_negated(m, kref);
        for (int j = j0; j < j1; ++j) {
            const bool iv = S.ivi[j] != 0;
            const int nv = m.nvert[j];
            cplx<float> ph, vl[4];
            proj_elem_data<float>(phi, vel, phi32, vel32, n, j, nv, iv, kref, neg, ph, vl);
            Elem32 e;
            load_elem32(mk, j, xhi, xlo, e);
            const float isq = m.isqa32[j];
            const float q2 = (e.D[0] * e.D[0] + e.D[1] * e.D[1] + e.D[2] * e.D[2]) * (isq * isq);
            bool near = false;
            int order = 2;
            if (q2 <= c_quad.far2_sq && !classify_fast(sqrtf(q2), near, order)) {
                const double xp[3] = {S.pts[3 * pp], S.pts[3 * pp + 1], S.pts[3 * pp + 2]};
                const double rd = ratio0_exact(mk, j, xp);
                near = rd < kTolf;
                if (!near) order = gauss_order(rd);
            }
            if (!near && e.nv == 3 && !iv) {
                float2 P = make_float2(0.f, 0.f), U[3], Tn = make_float2(0.f, 0.f);
                U[0] = U[1] = U[2] = make_float2(0.f, 0.f);
                const float dny = e.D[0] * e.n[0] + e.D[1] * e.n[1] + e.D[2] * e.n[2];
                if (order <= 2) proj_tri_points<4, 0>(e, dny, k2, wr, P, U, Tn);
                else if (order == 3) proj_tri_points<7, 4>(e, dny, k2, wr, P, U, Tn);
                else proj_tri_points<13, 11>(e, dny, k2, wr, P, U, Tn);
                const cplx<float> pq = ph * cplx<float>{P.x, P.y};
                acc.p.re += pq.re;
                acc.p.im += pq.im;
#pragma unroll
                for (int kk = 0; kk < 3; ++kk) {
                    const cplx<float> gg = ph * cplx<float>{fmaf(Tn.x, e.n[kk], U[kk].x), fmaf(Tn.y, e.n[kk], U[kk].y)};
                    acc.g[kk].re += gg.re;
                    acc.g[kk].im += gg.im;
                }
            } else if (!near) {
                const int np = e.nv == 3 ? tri_count(order) : quad_count(order);
                for (int gq = 0; gq < np; ++gq) {
                    float s, t, wq;
                    if (e.nv == 3) {
                        const int o = tri_offset(order) + gq;
                        s = c_trif[o][0]; t = c_trif[o][1]; wq = c_trif[o][2];
                    } else {
                        const int a = gq / order, b = gq - a * order;
                        s = c_glxf[order][a]; t = c_glxf[order][b];
                        wq = c_glwf[order][a] * c_glwf[order][b];
                    }
                    QPoint<float> q;
                    map_point(e, s, t, wq, q);
                    proj_point(q, ph, vl, e.nv, iv, k, wr, acc);
                }
            }
            // near pairs: the whole warp subdivides for one lane's point at a time
            unsigned todo = __ballot_sync(0xffffffffu, pv && near);
            if (todo) {
                Elem64 e64;
                load_elem64(mk, j, e64);
                cplx<float> phn, vln[4];
                proj_elem_data<float>(phi, vel, phi32, vel32, n, j, nv, true, kref, neg, phn, vln);
                while (todo) {
                    const int L = __ffs(todo) - 1;
                    todo &= todo - 1;
                    double xl[3];
                    float lh[3], ll[3];
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        xl[c] = S.pts[3 * (g * 32 + L) + c];   // lane L's point, a uniform load
                        lh[c] = __shfl_sync(0xffffffffu, xhi[c], L);
                        ll[c] = __shfl_sync(0xffffffffu, xlo[c], L);
                    }
                    Elem32 e32;
                    load_elem32(mk, j, lh, ll, e32);
                    ProjSink<float> sink;
                    sink.e = &e32; sink.phi = phn; sink.vel = vln; sink.ivi = iv; sink.k = k; sink.wr = wr;
                    sink.init();
                    const int rc = warp_subdivide(e64, m.area64[j], xl, ws, sink, &e32, isq);
                    if (rc != kDevOk) err = rc;
                    const ProjAcc<float> r = sink.reduce();
                    if (lane == L) {
                        acc.p += r.p;
                        for (int kk = 0; kk < 3; ++kk) acc.g[kk] += r.g[kk];
                    }
                }
            }
        }
    }
    float4 *out = S.part + 2 * ((size_t)(sl * G + g) * 32 + lane);
    out[0] = make_float4(acc.p.re, acc.p.im, acc.g[0].re, acc.g[0].im);
    out[1] = make_float4(acc.g[1].re, acc.g[1].im, acc.g[2].re, acc.g[2].im);
    if (err != kDevOk && lane == 0) atomicMax(S.status, err);
}

// Several right-hand sides of one matrix (bem_solve_multi): systems
// 0 .. nr-1 of the batch share the mesh, the points and the slicing and
// differ in their element data.  The pass over (32-point group, element
// slice) items is the one of k_project_pts, but a far flat triangle whose
// elements carry no velocity term in any right-hand side is evaluated once
// (P, U, T of proj_tri_points, independent of phi) and applied to every
// right-hand side's phi: the kernel evaluations, which dominate, are shared,
// and each right-hand side adds 4 complex multiply-adds per element.  Other
// pairs (velocity terms, quadrilaterals, subdivided near pairs) are evaluated
// per right-hand side as in k_project_pts.  Each right-hand side's partial
// sums go to its own scratch; k_project_sum finishes them.
// acc[r] += a with every index known at compile time (a runtime index
// would put the accumulators in local memory)
template <int RMAX>
__device__ __forceinline__ void acc_add(ProjAcc<float> (&acc)[RMAX], int r, const ProjAcc<float> &a) {
#pragma unroll
    for (int q = 0; q < RMAX; ++q)
        if (q == r) {
            acc[q].p += a.p;
#pragma unroll
            for (int kk = 0; kk < 3; ++kk) acc[q].g[kk] += a.g[kk];
        }
}

template <int RMAX>
__global__ void __launch_bounds__(256, RMAX <= 4 ? 2 : 1) k_project_pts_multi(const __grid_constant__ ProjBatch tb, int nr) {
    __shared__ WarpScratch ws_all[8];
    const ProjSys &S = tb.sys[0];
    const DevMesh m = to_dev(S.m);
    const DevFreq &f = S.f;
    const int lane = threadIdx.x, w = threadIdx.y, n = m.n, npts = S.npts;
    const int G = (npts + 31) >> 5, nsl = S.nslice;
    const int item = blockIdx.x * 8 + w;
    if (item >= G * nsl) return;
    const int g = item % G, sl = item / G;
    const int per = (n + nsl - 1) / nsl;
    const int j0 = sl * per, j1 = min(n, j0 + per);
    const int p = g * 32 + lane;
    const bool pv = p < npts;
    const int pp = pv ? p : g * 32;
    WarpScratch &ws = ws_all[w];
    float xhi[3], xlo[3];
    for (int c = 0; c < 3; ++c) {
        const double xv = S.pts[3 * pp + c];
        xhi[c] = (float)xv;
        xlo[c] = (float)(xv - (double)xhi[c]);
        asm volatile("" : "+f"(xhi[c]), "+f"(xlo[c]));
    }
    ProjAcc<float> acc[RMAX];
#pragma unroll
    for (int r = 0; r < RMAX; ++r) acc[r].p = acc[r].g[0] = acc[r].g[1] = acc[r].g[2] = cmk(0.f, 0.f);
    float k = (float)f.k, wr = (float)f.wr;
    asm volatile("" : "+f"(k), "+f"(wr));
    const float k2 = k * k;
    int err = kDevOk;
    for (int kref = 0; kref < m.sym.nref; ++kref) {
        const DevMesh mk = image_mesh(m, kref);
        const bool neg = image_negated(m, kref);
        for (int j = j0; j < j1; ++j) {
            bool iv_any = false;
#pragma unroll
            for (int r = 0; r < RMAX; ++r)
                if (r < nr && tb.sys[r].ivi[j] != 0) iv_any = true;
            const int nv = m.nvert[j];
            Elem32 e;
            load_elem32(mk, j, xhi, xlo, e);
            const float isq = m.isqa32[j];
            const float q2 = (e.D[0] * e.D[0] + e.D[1] * e.D[1] + e.D[2] * e.D[2]) * (isq * isq);
            bool near = false;
            int order = 2;
            if (q2 <= c_quad.far2_sq && !classify_fast(sqrtf(q2), near, order)) {
                const double xp[3] = {S.pts[3 * pp], S.pts[3 * pp + 1], S.pts[3 * pp + 2]};
                const double rd = ratio0_exact(mk, j, xp);
                near = rd < kTolf;
                if (!near) order = gauss_order(rd);
            }
            if (!near && e.nv == 3 && !iv_any) {
                float2 P = make_float2(0.f, 0.f), U[3], Tn = make_float2(0.f, 0.f);
                U[0] = U[1] = U[2] = make_float2(0.f, 0.f);
                const float dny = e.D[0] * e.n[0] + e.D[1] * e.n[1] + e.D[2] * e.n[2];
                if (order <= 2) proj_tri_points<4, 0>(e, dny, k2, wr, P, U, Tn);
                else if (order == 3) proj_tri_points<7, 4>(e, dny, k2, wr, P, U, Tn);
                else proj_tri_points<13, 11>(e, dny, k2, wr, P, U, Tn);
                cplx<float> gk[3];
#pragma unroll
                for (int kk = 0; kk < 3; ++kk) gk[kk] = cplx<float>{fmaf(Tn.x, e.n[kk], U[kk].x), fmaf(Tn.y, e.n[kk], U[kk].y)};
#pragma unroll
                for (int r = 0; r < RMAX; ++r) {
                    if (r >= nr) break;
                    const float2 p2 = ((const float2 *)tb.sys[r].phi32)[j];
                    const cplx<float> ph = neg ? cplx<float>{-p2.x, -p2.y} : cplx<float>{p2.x, p2.y};
                    const cplx<float> pq = ph * cplx<float>{P.x, P.y};
                    acc[r].p.re += pq.re;
                    acc[r].p.im += pq.im;
#pragma unroll
                    for (int kk = 0; kk < 3; ++kk) {
                        const cplx<float> gg = ph * gk[kk];
                        acc[r].g[kk].re += gg.re;
                        acc[r].g[kk].im += gg.im;
                    }
                }
            } else if (!near) {
                const int np = e.nv == 3 ? tri_count(order) : quad_count(order);
#pragma unroll 1
                for (int r = 0; r < RMAX; ++r) {
                    if (r >= nr) break;
                    const ProjSys &Sr = tb.sys[r];
                    const bool iv = Sr.ivi[j] != 0;
                    cplx<float> ph, vl[4];
                    proj_elem_data<float>((const double2 *)Sr.phi, (const double2 *)Sr.vel, (const float2 *)Sr.phi32,
                                          (const float2 *)Sr.vel32, n, j, nv, iv, kref, neg, ph, vl);
                    ProjAcc<float> tmp;
                    tmp.p = tmp.g[0] = tmp.g[1] = tmp.g[2] = cmk(0.f, 0.f);
                    for (int gq = 0; gq < np; ++gq) {
                        float s, t, wq;
                        if (e.nv == 3) {
                            const int o = tri_offset(order) + gq;
                            s = c_trif[o][0]; t = c_trif[o][1]; wq = c_trif[o][2];
                        } else {
                            const int a = gq / order, b = gq - a * order;
                            s = c_glxf[order][a]; t = c_glxf[order][b];
                            wq = c_glwf[order][a] * c_glwf[order][b];
                        }
                        QPoint<float> q;
                        map_point(e, s, t, wq, q);
                        proj_point(q, ph, vl, e.nv, iv, k, wr, tmp);
                    }
                    acc_add<RMAX>(acc, r, tmp);
                }
            }
            // near pairs: the whole warp subdivides for one lane's point at a
            // time, once per right-hand side
            unsigned todo = __ballot_sync(0xffffffffu, pv && near);
            if (todo) {
                Elem64 e64;
                load_elem64(mk, j, e64);
                while (todo) {
                    const int L = __ffs(todo) - 1;
                    todo &= todo - 1;
                    double xl[3];
                    float lh[3], ll[3];
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        xl[c] = S.pts[3 * (g * 32 + L) + c];
                        lh[c] = __shfl_sync(0xffffffffu, xhi[c], L);
                        ll[c] = __shfl_sync(0xffffffffu, xlo[c], L);
                    }
                    Elem32 e32;
                    load_elem32(mk, j, lh, ll, e32);
#pragma unroll 1
                    for (int r = 0; r < RMAX; ++r) {
                        if (r >= nr) break;
                        const ProjSys &Sr = tb.sys[r];
                        const bool iv = Sr.ivi[j] != 0;
                        cplx<float> phn, vln[4];
                        proj_elem_data<float>((const double2 *)Sr.phi, (const double2 *)Sr.vel,
                                              (const float2 *)Sr.phi32, (const float2 *)Sr.vel32, n, j, nv, true, kref,
                                              neg, phn, vln);
                        ProjSink<float> sink;
                        sink.e = &e32; sink.phi = phn; sink.vel = vln; sink.ivi = iv; sink.k = k; sink.wr = wr;
                        sink.init();
                        const int rc = warp_subdivide(e64, m.area64[j], xl, ws, sink, &e32, isq);
                        if (rc != kDevOk) err = rc;
                        const ProjAcc<float> rs = sink.reduce();
                        if (lane == L) acc_add<RMAX>(acc, r, rs);
                    }
                }
            }
        }
    }
#pragma unroll
    for (int r = 0; r < RMAX; ++r) {
        if (r >= nr) break;
        float4 *out = tb.sys[r].part + 2 * ((size_t)(sl * G + g) * 32 + lane);
        out[0] = make_float4(acc[r].p.re, acc[r].p.im, acc[r].g[0].re, acc[r].g[0].im);
        out[1] = make_float4(acc[r].g[1].re, acc[r].g[1].im, acc[r].g[2].re, acc[r].g[2].im);
    }
    if (err != kDevOk && lane == 0) atomicMax(S.status, err);
}

// Thread per point: the slices' partial sums in slice order (FP64), then the
// point's tau factor and incident field.
__global__ void __launch_bounds__(256) k_project_sum(const __grid_constant__ ProjBatch tb) {
    const int sb = find_sys(tb.ps_off, tb.B, blockIdx.x);
    const ProjSys &S = tb.sys[sb];
    const int p = (blockIdx.x - tb.ps_off[sb]) * 256 + threadIdx.x;
    if (p >= S.npts) return;
    const DevMesh m = to_dev(S.m);
    const int G = (S.npts + 31) >> 5;
    cplx<double> sp = {0.0, 0.0}, sg[3] = {{0.0, 0.0}, {0.0, 0.0}, {0.0, 0.0}};
    for (int sl = 0; sl < S.nslice; ++sl) {
        const float4 *in = S.part + 2 * ((size_t)sl * G * 32 + p);
        const float4 a = in[0], b = in[1];
        sp += cplx<double>{(double)a.x, (double)a.y};
        sg[0] += cplx<double>{(double)a.z, (double)a.w};
        sg[1] += cplx<double>{(double)b.x, (double)b.y};
        sg[2] += cplx<double>{(double)b.z, (double)b.w};
    }
    const double x64[3] = {S.pts[3 * p], S.pts[3 * p + 1], S.pts[3 * p + 2]};
    project_finish(m, S.f, x64, p, sp, sg, (double2 *)S.pot, (double2 *)S.grad);
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
    q.far2_sq = (float)((q.order_thr[2] * (1.0 + 3e-5)) * (q.order_thr[2] * (1.0 + 3e-5)));
    cudaError_t e = cudaMemcpyToSymbol(c_quad, &q, sizeof(q));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_trif, trif, sizeof(trif));
    float far4[4][4];
    for (int g = 0; g < 4; ++g) {
        far4[g][0] = trif[g][0] - (1.0f / 3.0f);
        far4[g][1] = trif[g][1] - (1.0f / 3.0f);
        far4[g][2] = 2.0f * far4[g][0];
        far4[g][3] = 2.0f * far4[g][1];
    }
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_far4, far4, sizeof(far4));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_glxf, glxf, sizeof(glxf));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_glwf, glwf, sizeof(glwf));
    return e;
}

cudaError_t launch_image_tables(const DevMeshView &m, const ImageTables &out, cudaStream_t st) {
    const long long total = (long long)(m.sym.nref - 1) * m.n;
    if (total <= 0) return cudaSuccess;
    count_launches(1);
    k_image_tables<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(m, out);
    return cudaGetLastError();
}

size_t near_list_scratch_bytes(int n, int nref) {
    const size_t nb = (size_t)(n + 31) / 32;
    return nb * (size_t)nref * sizeof(float4) + nb * sizeof(float);
}

cudaError_t launch_near_list(const DevMeshView &m, void *scratch, int2 *list, unsigned long long cap,
                             unsigned long long *count, cudaStream_t st) {
    const int nb = (m.n + 31) / 32;
    float4 *sph = (float4 *)scratch;
    float *bsq = (float *)(sph + (size_t)nb * m.sym.nref);
    dim3 block(32, 8);
    count_launches(2);
    k_block_spheres<<<(nb * m.sym.nref + 7) / 8, block, 0, st>>>(m, sph, bsq);
    k_near_list<<<(m.n + 7) / 8, block, 0, st>>>(m, sph, bsq, list, count, cap);
    return cudaGetLastError();
}

void asm_batch_finish(AsmBatch &t) {
    t.far_off[0] = t.near_off[0] = t.rhs_off[0] = 0;
    t.img = 0;
    for (int b = 0; b < t.B; ++b) {
        if (t.sys[b].m.sym.nref > 1) t.img = 1;
        const int n = t.sys[b].m.n;
        const int nt = (n + 31) / 32;
        t.far_off[b + 1] = t.far_off[b] + nt * ((n + 8 * kRowsPerThread - 1) / (8 * kRowsPerThread));
        t.near_off[b + 1] = t.near_off[b] + (int)t.sys[b].n_near;
        t.rhs_off[b + 1] = t.rhs_off[b] + (n + 7) / 8;
    }
}

void proj_batch_finish(ProjBatch &t) {
    t.fld_off[0] = t.pt_off[0] = t.lp_off[0] = t.ps_off[0] = 0;
    for (int b = 0; b < t.B; ++b) {
        ProjSys &S = t.sys[b];
        t.fld_off[b + 1] = t.fld_off[b] + (S.m.n + 255) / 256;
        t.pt_off[b + 1] = t.pt_off[b] + (S.npts + 7) / 8;
        // element slices of the float projection, as many as the scratch holds
        const long long G = (S.npts + 31) / 32;
        const long long want = (S.m.n + kProjSlice - 1) / kProjSlice;
        const long long fit = G > 0 ? S.part_cap / (2 * 32 * G) : 0;
        S.nslice = S.part ? (int)std::min(want, fit) : 0;
        t.lp_off[b + 1] = t.lp_off[b] + (int)((G * S.nslice + 7) / 8);
        t.ps_off[b + 1] = t.ps_off[b] + (S.npts + 255) / 256;
    }
}

namespace {
int g_sms = 0;
int sm_count() {
    if (g_sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
        if (g_sms <= 0) g_sms = 1;
    }
    return g_sms;
}
}  // namespace

cudaError_t launch_assemble(const AsmBatch &t, int prec, unsigned *ctr, cudaStream_t st, AsmShape shape) {
    if (t.B <= 0) return cudaSuccess;
    dim3 block(32, 8);
    const int far_items = t.far_off[t.B], near_items = t.near_off[t.B];
    // persistent grids: far_per_sm resident blocks of k_far per SM (launch
    // bounds allow kFarPerSm), near_per_sm of k_near (launch bounds allow 2)
    const int fps = std::max(1, std::min(shape.far_per_sm, kFarPerSm));
    const int nps = std::max(1, std::min(shape.near_per_sm, 2));
    const int gfar = std::max(1, std::min(far_items, fps * sm_count()));
    const int gnear = std::max(1, std::min((near_items + 7) / 8, nps * sm_count()));
    // Systems that fill the GPU on their own take one single-system launch
    // each: the single-system kernel keeps the table in constant operands
    // (fewer registers, no spills), which beat the shared work queue.
    bool split = t.B > 1;
    for (int b = 0; b < t.B && split; ++b)
        if (t.far_off[b + 1] - t.far_off[b] < fps * sm_count()) split = false;
    std::unique_ptr<AsmBatch> one_sys;
    if (split) one_sys.reset(new AsmBatch());
    count_launches((split ? t.B : 1) + (near_items ? 1 : 0));
    auto far = [&](const AsmBatch &a, int grid) {
        const bool one = a.B == 1;
        if (prec == 0) {
            if (a.img) {
                if (one) k_far<double, true, true><<<grid, block, 0, st>>>(a, ctr);
                else k_far<double, false, true><<<grid, block, 0, st>>>(a, ctr);
            } else {
                if (one) k_far<double, true, false><<<grid, block, 0, st>>>(a, ctr);
                else k_far<double, false, false><<<grid, block, 0, st>>>(a, ctr);
            }
        } else {
            if (a.img) {
                if (one) k_far<float, true, true><<<grid, block, 0, st>>>(a, ctr);
                else k_far<float, false, true><<<grid, block, 0, st>>>(a, ctr);
            } else {
                if (one) k_far<float, true, false><<<grid, block, 0, st>>>(a, ctr);
                else k_far<float, false, false><<<grid, block, 0, st>>>(a, ctr);
            }
        }
    };
    if (split) {
        // launches run in order on st; each ends by resetting the queue counter
        for (int b = 0; b < t.B; ++b) {
            one_sys->B = 1;
            one_sys->sys[0] = t.sys[b];
            asm_batch_finish(*one_sys);
            far(*one_sys, std::max(1, std::min(one_sys->far_off[1], fps * sm_count())));
        }
    } else {
        far(t, gfar);
    }
    if (near_items) {
        if (prec == 0) k_near<double><<<gnear, block, 0, st>>>(t, ctr + 2);
        else k_near<float><<<gnear, block, 0, st>>>(t, ctr + 2);
    }
    return cudaGetLastError();
}

cudaError_t launch_rhs(const AsmBatch &t, cudaStream_t st) {
    if (t.B <= 0) return cudaSuccess;
    dim3 block(32, 8);
    count_launches(1);
    k_rhs<<<t.rhs_off[t.B], block, 0, st>>>(t);
    return cudaGetLastError();
}

cudaError_t launch_fields(const ProjBatch &t, cudaStream_t st) {
    if (t.B <= 0 || t.fld_off[t.B] == 0) return cudaSuccess;
    count_launches(1);
    k_fields<<<t.fld_off[t.B], 256, 0, st>>>(t);
    return cudaGetLastError();
}

cudaError_t launch_project_multi(const ProjBatch &t, cudaStream_t st) {
    // the right-hand sides of one solver: same mesh, points and slicing
    bool shared = t.B >= 2 && t.B <= 8 && t.sys[0].nslice > 0;
    for (int b = 1; b < t.B && shared; ++b)
        shared = t.sys[b].npts == t.sys[0].npts && t.sys[b].pts == t.sys[0].pts &&
                 t.sys[b].nslice == t.sys[0].nslice && t.sys[b].m.n == t.sys[0].m.n;
    if (!shared) return launch_project(t, 1, st);
    if (t.sys[0].npts == 0) return cudaSuccess;
    dim3 block(32, 8);
    const int items = ((t.sys[0].npts + 31) / 32) * t.sys[0].nslice;
    const int grid = (items + 7) / 8;
    count_launches(2);
    if (t.B <= 2) k_project_pts_multi<2><<<grid, block, 0, st>>>(t, t.B);
    else if (t.B <= 4) k_project_pts_multi<4><<<grid, block, 0, st>>>(t, t.B);
    else k_project_pts_multi<8><<<grid, block, 0, st>>>(t, t.B);
    k_project_sum<<<t.ps_off[t.B], 256, 0, st>>>(t);
    return cudaGetLastError();
}

cudaError_t launch_project(const ProjBatch &t, int prec, cudaStream_t st) {
    if (t.B <= 0 || t.pt_off[t.B] == 0) return cudaSuccess;
    dim3 block(32, 8);
    bool sliced = prec != 0;
    for (int b = 0; b < t.B; ++b)
        if (t.sys[b].npts > 0 && t.sys[b].nslice == 0) sliced = false;   // scratch too short
    if (prec == 0) {
        count_launches(1);
        k_project<double><<<t.pt_off[t.B], block, 0, st>>>(t);
    } else if (!sliced) {
        count_launches(1);
        k_project<float><<<t.pt_off[t.B], block, 0, st>>>(t);
    } else {
        count_launches(2);
        k_project_pts<<<t.lp_off[t.B], block, 0, st>>>(t);
        k_project_sum<<<t.ps_off[t.B], 256, 0, st>>>(t);
    }
    return cudaGetLastError();
}

}  // namespace bem
