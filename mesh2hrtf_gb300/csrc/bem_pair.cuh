// bem_pair.cuh - warp-cooperative integration of one (point, element) pair
// with NumCalc's adaptive subdivision, the singular self-element integral,
// and the sinks that turn quadrature points into matrix entries, right-hand
// side terms or field values.
#pragma once

#include "bem_common.cuh"

namespace bem {

// Per-warp scratch in shared memory.  Subelement vertex coordinates are
// dyadic fractions of the parent's local coordinates in [-1, 1]; float holds
// them exactly up to kMaxLevel halvings.  Deeper subdivision only happens for
// points within ~1e-7 element sizes of the surface, where NumCalc itself ends
// with its subelement-count error; the kernels report the same error.
struct WarpScratch {
    float lv[2][kMaxLevelSub][4][2];   // [level parity][subelement][vertex][s,t]
    float sxi[32], seta[32], sfac[32]; // stored subelements of the current chunk
    int sord[32];
    int soff[33];
};

// ---------------------------------------------------------------- sinks
// Assembly: accumulate G, H, H^T, E of the pair in precision T.
template <typename T> struct AsmSink;

template <> struct AsmSink<double> {
    static constexpr bool kFloatPoints = false;   // quadrature points in FP64
    const Elem64 *e;
    const double *x, *nx;
    double k, wr;
    KVals<double> acc;
    __device__ void init() { acc.G = acc.H = acc.HT = acc.E = cmk(0.0, 0.0); }
    __device__ void add(double s, double t, double w) {
        QPoint<double> q;
        map_point(*e, s, t, x, w, q);
        KVals<double> v = kernel_values(q, nx, k, wr);
        acc.G += v.G; acc.H += v.H; acc.HT += v.HT; acc.E += v.E;
    }
    __device__ KVals<double> reduce() {
        return {warp_sum(acc.G), warp_sum(acc.H), warp_sum(acc.HT), warp_sum(acc.E)};
    }
};

template <> struct AsmSink<float> {
    static constexpr bool kFloatPoints = true;    // quadrature points in float (addf)
    const Elem32 *e;
    const float *nx;
    float k, wr;
    KVals<float> acc;
    __device__ void init() { acc.G = acc.H = acc.HT = acc.E = cmk(0.f, 0.f); }
    __device__ void addf(float s, float t, float w) {
        QPoint<float> q;
        map_point(*e, s, t, w, q);
        KVals<float> v = kernel_values(q, nx, k, wr);
        acc.G += v.G; acc.H += v.H; acc.HT += v.HT; acc.E += v.E;
    }
    __device__ void add(double s, double t, double w) { addf((float)s, (float)t, (float)w); }
    __device__ KVals<float> reduce() {
        return {warp_sum(acc.G), warp_sum(acc.H), warp_sum(acc.HT), warp_sum(acc.E)};
    }
};

// Right-hand side contribution of a column with prescribed nonzero boundary
// values (Zrsintel[4] of NC_RegularIntegration, NC_EquationSystem.cpp:1719-1725).
struct RhsSink {
    static constexpr bool kFloatPoints = false;
    const Elem64 *e;
    const double *x, *nx;
    const cplx<double> *bc;   // nodal values
    int bctype;               // 0 velocity (also with admittance), 1 pressure
    Phys<double> P;
    cplx<double> acc;
    __device__ void init() { acc = cmk(0.0, 0.0); }
    __device__ void add(double s, double t, double w) {
        QPoint<double> q;
        map_point(*e, s, t, x, w, q);
        KVals<double> v = kernel_values(q, nx, P.k, P.wr);
        cplx<double> bcv = cmk(0.0, 0.0);
        for (int a = 0; a < e->nv; ++a) bcv += bc[a] * q.sh[a];
        cplx<double> beta = {0.0, P.beta_im};
        if (bctype == 0) acc += (v.G * P.tao + v.HT * beta) * bcv;
        else acc -= (v.H * P.tao + v.E * beta) * bcv;
    }
    __device__ cplx<double> reduce() { return warp_sum(acc); }
};

// Field projection (NC_IntegrationTBEM, NC_PostProcessing.cpp:1217-1322):
// potential and gradient at x from the element potential phi and the nodal
// normal velocities vel.
template <typename T> struct ProjAcc { cplx<T> p, g[3]; };

template <typename T>
__device__ __forceinline__ void proj_point(const QPoint<T> &q, cplx<T> phi, const cplx<T> *vel, int nv,
                                           bool ivi, T k, T wr, ProjAcc<T> &a) {
    const T r = q.r, ir = q.ir;
    T dh[3] = {q.d[0] * ir, q.d[1] * ir, q.d[2] * ir};
    T s, c;
    sincos_t(wr * r, &s, &c);
    T amp = T(1.0 / kPI4) * ir;
    cplx<T> zgr = {c * amp, s * amp};
    cplx<T> zgikr = zgr * cplx<T>{-ir, wr};
    T drdnx = dh[0] * q.ny[0] + dh[1] * q.ny[1] + dh[2] * q.ny[2];
    cplx<T> zfac1 = zgr * cplx<T>{drdnx * (k * k - T(3) * ir * ir), wr * T(3) * drdnx * ir};
    cplx<T> zfac2 = zgikr * (-ir);
    cplx<T> z1 = phi * q.wj;
    a.p += (zgikr * drdnx) * z1;
#pragma unroll
    for (int kk = 0; kk < 3; ++kk) a.g[kk] += (zfac1 * dh[kk] + zfac2 * q.ny[kk]) * z1;
    if (ivi) {
        for (int v = 0; v < nv; ++v) {
            cplx<T> zz = vel[v] * (q.wj * q.sh[v]);
            a.p -= zgr * zz;
#pragma unroll
            for (int kk = 0; kk < 3; ++kk) a.g[kk] -= (zgikr * (-dh[kk])) * zz;
        }
    }
}

template <typename T> struct ProjSink;

template <> struct ProjSink<double> {
    static constexpr bool kFloatPoints = false;
    const Elem64 *e;
    const double *x;
    cplx<double> phi;
    const cplx<double> *vel;
    bool ivi;
    double k, wr;
    ProjAcc<double> acc;
    __device__ void init() { acc.p = acc.g[0] = acc.g[1] = acc.g[2] = cmk(0.0, 0.0); }
    __device__ void add(double s, double t, double w) {
        QPoint<double> q;
        map_point(*e, s, t, x, w, q);
        proj_point(q, phi, vel, e->nv, ivi, k, wr, acc);
    }
    __device__ ProjAcc<double> reduce() {
        ProjAcc<double> r;
        r.p = warp_sum(acc.p);
        for (int kk = 0; kk < 3; ++kk) r.g[kk] = warp_sum(acc.g[kk]);
        return r;
    }
};

template <> struct ProjSink<float> {
    static constexpr bool kFloatPoints = true;
    const Elem32 *e;
    cplx<float> phi;
    const cplx<float> *vel;
    bool ivi;
    float k, wr;
    ProjAcc<float> acc;
    __device__ void init() { acc.p = acc.g[0] = acc.g[1] = acc.g[2] = cmk(0.f, 0.f); }
    __device__ void addf(float s, float t, float w) {
        QPoint<float> q;
        map_point(*e, s, t, w, q);
        proj_point(q, phi, vel, e->nv, ivi, k, wr, acc);
    }
    __device__ void add(double s, double t, double w) { addf((float)s, (float)t, (float)w); }
    __device__ ProjAcc<float> reduce() {
        ProjAcc<float> r;
        r.p = warp_sum(acc.p);
        for (int kk = 0; kk < 3; ++kk) r.g[kk] = warp_sum(acc.g[kk]);
        return r;
    }
};

// ------------------------------------------------- local quadrature points
// Point g of a stored subelement (origin xice/etce, signed scale fase,
// order): NC_RegularIntegration, NC_EquationSystem.cpp:1654-1683.
__device__ __forceinline__ void sub_point(int nv, int order, int g, double xice, double etce, double fase,
                                          double &s, double &t, double &w) {
    double cs, ct, cw;
    if (nv == 3) {
        const int o = tri_offset(order) + g;
        cs = c_quad.tri[o][0]; ct = c_quad.tri[o][1]; cw = c_quad.tri[o][2];
    } else {
        const int i = g / order, jj = g - i * order;
        cs = c_quad.glx[order][i]; ct = c_quad.glx[order][jj];
        cw = c_quad.glw[order][i] * c_quad.glw[order][jj];
    }
    if (fabs(fase - 1.0) < kEPSY) { s = cs; t = ct; w = cw; }
    else { s = xice + cs * fase; t = etce + ct * fase; w = cw * (fase * fase); }
}

// The same in float for the float sinks: the stored origin and scale are
// exact floats (dyadic), the rule's tables float; the point moves by float
// rounding only (~1e-7 of the element), below the float kernel arithmetic.
__device__ __forceinline__ void sub_point_f(int nv, int order, int g, float xice, float etce, float fase,
                                            float &s, float &t, float &w) {
    float cs, ct, cw;
    if (nv == 3) {
        const int o = tri_offset(order) + g;
        cs = c_trif[o][0]; ct = c_trif[o][1]; cw = c_trif[o][2];
    } else {
        const int i = g / order, jj = g - i * order;
        cs = c_glxf[order][i]; ct = c_glxf[order][jj];
        cw = c_glwf[order][i] * c_glwf[order][jj];
    }
    if (fase == 1.0f) { s = cs; t = ct; w = cw; }   // |fase - 1| < 1e-14 for dyadic fase
    else { s = fmaf(cs, fase, xice); t = fmaf(ct, fase, etce); w = cw * (fase * fase); }
}

__device__ __forceinline__ int sub_npts(int nv, int order) {
    return nv == 3 ? tri_count(order) : quad_count(order);
}

// ------------------------------------------------------ subdivision (warp)
// NC_GenerateSubelements (NC_3dFunctions.cpp:575-783) executed by a whole
// warp: the subelements of one level are classified in parallel, split ones
// get their children in the reference's order via ballot ranks, and the
// stored ones are integrated immediately (points spread over the lanes).
// Returns kDevOk or an error code; all lanes return the same value and every
// lane's sink holds a partial sum (the caller reduces).
// Fast decisions: with ef (the element's float tables for this point, D =
// centre - x in double-float) and isqa = 1/sqrt(area) in float, levels up to
// kFastLevels decide "split" and the Gauss order from a float ratio, and take
// the exact FP64 test only within 2e-5 of a threshold; deeper levels (points
// within an eighth of the element from it) always take the exact test.  The
// decisions are the exact ones either way: the float ratio is accurate to
// ~1e-6 relative there.
constexpr int kFastLevels = 3;

template <class Sink>
__device__ int warp_subdivide(const Elem64 &e, double area, const double x[3], WarpScratch &ws, Sink &sink,
                              const Elem32 *ef = nullptr, float isqa = 0.f) {
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const int nv = e.nv;
    if (lane < nv) {
        ws.lv[0][0][lane][0] = nv == 3 ? c_csi6f[lane] : c_csi8f[lane];
        ws.lv[0][0][lane][1] = nv == 3 ? c_eta6f[lane] : c_eta8f[lane];
    }
    __syncwarp();
    int cur = 0, nsel = 1, nsbe = 0, err = kDevOk;
    // NumCalc's sqrt(area faclin^2) equals sqrt(area) faclin exactly (faclin
    // is a power of two): one FP64 square root per pair, not per level
    const double sqa0 = __dsqrt_rn(area);
    double faclin = 2.0;
    for (int level = 0; level <= kMaxLevel; ++level) {
        faclin *= 0.5;
        const float faclinf = (float)faclin;   // a power of two
        int ndie = 0;
        for (int base = 0; base < nsel; base += 32) {
            const int idi = base + lane;
            const bool active = idi < nsel;
            bool split = false;
            int ordf = 0;   // Gauss order from the float test (0: not decided there)
            double ratdis = 0.0, scent = 0.0, tcent = 0.0;
            // vertices as stored (exact floats); FP64 copies only where the
            // exact arithmetic needs them
            float vsf[4] = {0.f, 0.f, 0.f, 0.f}, vtf[4] = {0.f, 0.f, 0.f, 0.f};
            if (active) {
                for (int v = 0; v < nv; ++v) {
                    vsf[v] = ws.lv[cur][idi][v][0];
                    vtf[v] = ws.lv[cur][idi][v][1];
                }
                bool decided = false;
                if (ef && level <= kFastLevels) {
                    float sc = 0.f, tc = 0.f;
                    for (int v = 0; v < nv; ++v) {
                        sc += vsf[v];
                        tc += vtf[v];
                    }
                    sc /= (float)nv;
                    tc /= (float)nv;
                    float d[3];
                    if (nv == 3) {
                        const float ss = sc - (1.0f / 3.0f), tt = tc - (1.0f / 3.0f);
                        for (int k = 0; k < 3; ++k) d[k] = ef->D[k] + ss * ef->a[k] + tt * ef->b[k];
                    } else {
                        const float s1 = 0.25f * (sc + 1.0f), s2 = 0.25f * (sc - 1.0f), t1 = tc + 1.0f, t2 = tc - 1.0f;
                        const float sh[4] = {s1 * t1, -s2 * t1, s2 * t2, -s1 * t2};
                        for (int k = 0; k < 3; ++k)
                            d[k] = ef->D[k] + sh[0] * ef->q[0][k] + sh[1] * ef->q[1][k] + sh[2] * ef->q[2][k] +
                                   sh[3] * ef->q[3][k];
                    }
                    const float rf = sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) * isqa / faclinf;
                    bool nr = false;
                    int o = 2;
                    if (classify_fast(rf, nr, o)) {
                        split = nr;
                        ordf = nr ? 0 : o;
                        decided = true;
                    }
                }
                // the FP64 centre: for the exact test, and for the children of
                // a split quadrilateral (the centre is one of their vertices)
                if (!decided || (split && nv == 4)) {
                    for (int v = 0; v < nv; ++v) {
                        scent = __dadd_rn(scent, (double)vsf[v]);
                        tcent = __dadd_rn(tcent, (double)vtf[v]);
                    }
                    scent = __ddiv_rn(scent, (double)nv);
                    tcent = __ddiv_rn(tcent, (double)nv);
                }
                if (!decided) {
                    double cp[3];
                    global_point_exact(e, scent, tcent, cp);
                    ratdis = __ddiv_rn(dist_exact(cp, x), __dmul_rn(sqa0, faclin));
                    split = ratdis < kTolf;
                }
            }
            const unsigned smask = __ballot_sync(0xffffffffu, split);
            if (split) {
                const int rank = ndie + __popc(smask & lt);   // 0-based count of earlier splits
                if (rank + 1 > 15) {
                    err = kDevSplitLimit;
                } else {
                    // midpoints of dyadic vertices: exact in float
                    float ms[8], mt[8];
                    for (int v = 0; v < nv; ++v) {
                        int v1 = v + 1 == nv ? 0 : v + 1;
                        ms[v] = vsf[v]; mt[v] = vtf[v];
                        ms[v + nv] = (vsf[v] + vsf[v1]) * 0.5f;
                        mt[v + nv] = (vtf[v] + vtf[v1]) * 0.5f;
                    }
                    const int nxt = cur ^ 1, c0 = rank * 4;
                    for (int v = 0; v < nv; ++v) {
                        const int nsu = c0 + v, j1 = v + nv;
                        int j2 = j1 - 1;
                        if (j2 < nv) j2 += nv;
                        ws.lv[nxt][nsu][0][0] = ms[v];  ws.lv[nxt][nsu][0][1] = mt[v];
                        ws.lv[nxt][nsu][1][0] = ms[j1]; ws.lv[nxt][nsu][1][1] = mt[j1];
                        if (nv == 4) {
                            ws.lv[nxt][nsu][2][0] = (float)scent;  ws.lv[nxt][nsu][2][1] = (float)tcent;
                            ws.lv[nxt][nsu][3][0] = ms[j2]; ws.lv[nxt][nsu][3][1] = mt[j2];
                        } else {
                            ws.lv[nxt][nsu][2][0] = ms[j2]; ws.lv[nxt][nsu][2][1] = mt[j2];
                            ws.lv[nxt][c0 + 3][v][0] = ms[j1];
                            ws.lv[nxt][c0 + 3][v][1] = mt[j1];
                        }
                    }
                }
            }
            ndie += __popc(smask);
            const bool store = active && !split;
            const unsigned stmask = __ballot_sync(0xffffffffu, store);
            const int nst = __popc(stmask);
            if (store) {
                const int r = __popc(stmask & lt);
                if (nsbe + r >= kMSBE) err = kDevSubLimit;
                float ox, oy, fac;
                if (nv == 4) {
                    const double vs[4] = {vsf[0], vsf[1], vsf[2], vsf[3]}, vt[4] = {vtf[0], vtf[1], vtf[2], vtf[3]};
                    ox = (float)((vs[0] + vs[1] + vs[2] + vs[3]) / 4.0);
                    oy = (float)((vt[0] + vt[1] + vt[2] + vt[3]) / 4.0);
                    fac = faclinf;
                } else {
                    // the vertex whose offset to the centroid is equal in s and
                    // t (NC_GenerateSubelements): with dyadic vertices the sums
                    // and 3 v are exact in float, so the reference's test
                    // |(c_s - s_v) - (c_t - t_v)| < 1e-8 is exact equality here
                    const float ssum = vsf[0] + vsf[1] + vsf[2], tsum = vtf[0] + vtf[1] + vtf[2];
                    int jr = 0;
                    float dxi = 0.f;
                    for (int v = 0; v < 3; ++v) {
                        dxi = ssum - 3.f * vsf[v];
                        const float det = tsum - 3.f * vtf[v];
                        if (dxi == det) { jr = v; break; }
                    }
                    ox = vsf[jr]; oy = vtf[jr];
                    fac = dxi >= 0.f ? faclinf : -faclinf;
                }
                const int ord = ordf ? ordf : gauss_order(ratdis);
                ws.sxi[r] = ox; ws.seta[r] = oy; ws.sfac[r] = fac;
                ws.sord[r] = ord;
            }
            __syncwarp();
            // offsets of the stored subelements' points; ranks are dense 0..nst-1
            int incl = lane < nst ? sub_npts(nv, ws.sord[lane]) : 0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += y;
            }
            ws.soff[lane + 1] = incl;
            if (lane == 0) ws.soff[0] = 0;
            __syncwarp();
            const int total = ws.soff[nst];
            for (int f = lane; f < total; f += 32) {
                int sidx = 0;
                while (ws.soff[sidx + 1] <= f) ++sidx;
                const int g = f - ws.soff[sidx];
                if constexpr (Sink::kFloatPoints) {
                    float s, t, w;
                    sub_point_f(nv, ws.sord[sidx], g, ws.sxi[sidx], ws.seta[sidx], ws.sfac[sidx], s, t, w);
                    sink.addf(s, t, w);
                } else {
                    double s, t, w;
                    sub_point(nv, ws.sord[sidx], g, (double)ws.sxi[sidx], (double)ws.seta[sidx],
                              (double)ws.sfac[sidx], s, t, w);
                    sink.add(s, t, w);
                }
            }
            nsbe += nst;
            __syncwarp();
        }
        err = __reduce_max_sync(0xffffffffu, err);
        if (err != kDevOk) return err;
        if (ndie == 0) return kDevOk;
        nsel = ndie * 4;
        cur ^= 1;
        __syncwarp();
    }
    return kDevSplitLimit;
}

// ------------------------------------------------------ singular (warp)
// Self-element integrals in FP64 (NC_SingularIntegration,
// NC_EquationSystem.cpp:1408-1597): the hypersingular part of E by Stokes'
// theorem as edge integrals (4 sections x 3 Gauss points per edge), G, H,
// H^T and the k^2 part of E over 2 sub-triangles per edge from the centre
// with a collapsed 4x4 Gauss rule.  Points are spread over the lanes.
struct SingOut {
    KVals<double> v;
    cplx<double> rhs;   // Zrsintel[4]
};

__device__ __forceinline__ SingOut warp_singular(const Elem64 &e, const double x[3], const double nx[3],
                                                 const Phys<double> &P, int rhs_mode,
                                                 const cplx<double> *bc) {
    // rhs_mode: 0 none, 1 velocity values, 2 pressure values
    const int lane = threadIdx.x & 31;
    const int nv = e.nv;
    const double wnu2 = P.k * P.k;
    const cplx<double> beta = {0.0, P.beta_im};
    cplx<double> zG = cmk(0.0, 0.0), zH = zG, zHT = zG, zE = zG, zR = zG;
    const int n_edge = nv * 12, n_area = nv * 32;
    // 3-point Gauss on [-1, 1]
    for (int f = lane; f < n_edge + n_area; f += 32) {
        if (f < n_edge) {
            const int ieg = f / 12, rem = f - ieg * 12, isec = rem / 3, ig = rem - isec * 3;
            const int ig1 = ieg + 1 == nv ? 0 : ieg + 1;
            double dif[3], len = 0.0;
            for (int k = 0; k < 3; ++k) { dif[k] = e.p[ig1][k] - e.p[ieg][k]; len += dif[k] * dif[k]; }
            len = sqrt(len);
            double dio[3] = {dif[0] / len, dif[1] / len, dif[2] / len};
            const double leneg = len / 8.0;
            const double secmid = -0.75 + 0.5 * (double)isec;
            const double sga = secmid + c_quad.glx[3][ig] / 4.0;
            const double wga = c_quad.glw[3][ig] * leneg;
            double d[3];
            for (int k = 0; k < 3; ++k) d[k] = (e.p[ieg][k] + dif[k] * (sga + 1.0) / 2.0) - x[k];
            const double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            for (int k = 0; k < 3; ++k) d[k] /= r;
            double sn, cs;
            sincos(P.wr * r, &sn, &cs);
            cplx<double> zg = cmk(cs / (kPI4 * r), sn / (kPI4 * r)) * cmk(-1.0 / r, P.wr);
            cplx<double> g0 = zg * d[0], g1 = zg * d[1], g2 = zg * d[2];
            cplx<double> w0 = g1 * dio[2] - g2 * dio[1];
            cplx<double> w1 = g2 * dio[0] - g0 * dio[2];
            cplx<double> w2 = g0 * dio[1] - g1 * dio[0];
            zE += (w0 * nx[0] + w1 * nx[1] + w2 * nx[2]) * wga;
        } else {
            const int fa = f - n_edge;
            const int ieg = fa / 32, rem = fa - ieg * 32, isec = rem / 16, g = rem - isec * 16;
            const int ig1 = ieg + 1 == nv ? 0 : ieg + 1, ig2 = ieg + nv;
            double ss[3], ts[3], aresub;
            if (nv == 3) {
                aresub = 1.0 / 24.0 / 2.0;
                ss[0] = ts[0] = 1.0 / 3.0;
                if (isec == 0) { ss[1] = c_csi6[ieg]; ss[2] = c_csi6[ig2]; ts[1] = c_eta6[ieg]; ts[2] = c_eta6[ig2]; }
                else { ss[1] = c_csi6[ig2]; ss[2] = c_csi6[ig1]; ts[1] = c_eta6[ig2]; ts[2] = c_eta6[ig1]; }
            } else {
                aresub = 0.25 / 2.0;
                ss[0] = ts[0] = 0.0;
                if (isec == 0) { ss[1] = c_csi8[ieg]; ss[2] = c_csi8[ig2]; ts[1] = c_eta8[ieg]; ts[2] = c_eta8[ig2]; }
                else { ss[1] = c_csi8[ig2]; ss[2] = c_csi8[ig1]; ts[1] = c_eta8[ig2]; ts[2] = c_eta8[ig1]; }
            }
            const int gi = g / 4, gj = g - gi * 4;
            const double sga = c_quad.glx[4][gi], tga = c_quad.glx[4][gj];
            const double wq = c_quad.glw[4][gi] * c_quad.glw[4][gj];
            const double sgg = 0.5 * (1.0 - sga) * ss[0] + 0.25 * (1.0 + sga) * ((1.0 - tga) * ss[1] + (1.0 + tga) * ss[2]);
            const double tgg = 0.5 * (1.0 - sga) * ts[0] + 0.25 * (1.0 + sga) * ((1.0 - tga) * ts[1] + (1.0 + tga) * ts[2]);
            QPoint<double> q;
            map_point(e, sgg, tgg, x, wq * (1.0 + sga) * aresub, q);
            const double r = q.r;
            double dh[3] = {q.d[0] / r, q.d[1] / r, q.d[2] / r};
            double sn, cs;
            sincos(P.wr * r, &sn, &cs);
            const double re2 = q.wj / kPI4 / r;
            cplx<double> zg = cmk(cs * re2, sn * re2);
            cplx<double> zh = zg * cmk(-1.0 / r, P.wr);
            const double re1 = dh[0] * q.ny[0] + dh[1] * q.ny[1] + dh[2] * q.ny[2];
            const double rr2 = -(dh[0] * nx[0] + dh[1] * nx[1] + dh[2] * nx[2]);
            cplx<double> zhh = zh * re1, zht = zh * rr2;
            zG += zg; zH += zhh; zHT += zht;
            zE += zg * (wnu2 * (nx[0] * q.ny[0] + nx[1] * q.ny[1] + nx[2] * q.ny[2]));
            if (rhs_mode == 1) {
                cplx<double> bcv = cmk(0.0, 0.0);
                for (int a = 0; a < nv; ++a) bcv += bc[a] * q.sh[a];
                zR += (zg * P.tao + zht * beta) * bcv;
            }
        }
    }
    SingOut o;
    o.v.G = warp_sum(zG); o.v.H = warp_sum(zH); o.v.HT = warp_sum(zHT); o.v.E = warp_sum(zE);
    o.rhs = warp_sum(zR);
    if (rhs_mode == 2) {
        // pressure values: -(H tao + E beta) * value at the last area point
        // (edge nv-1, second sub-triangle, Gauss point 15), NC_EquationSystem.cpp:1592-1596
        const int ieg = nv - 1, ig1 = 0, ig2 = ieg + nv;
        double ss[3], ts[3];
        if (nv == 3) { ss[0] = ts[0] = 1.0 / 3.0; ss[1] = c_csi6[ig2]; ss[2] = c_csi6[ig1]; ts[1] = c_eta6[ig2]; ts[2] = c_eta6[ig1]; }
        else { ss[0] = ts[0] = 0.0; ss[1] = c_csi8[ig2]; ss[2] = c_csi8[ig1]; ts[1] = c_eta8[ig2]; ts[2] = c_eta8[ig1]; }
        const double sga = c_quad.glx[4][3], tga = c_quad.glx[4][3];
        const double sgg = 0.5 * (1.0 - sga) * ss[0] + 0.25 * (1.0 + sga) * ((1.0 - tga) * ss[1] + (1.0 + tga) * ss[2]);
        const double tgg = 0.5 * (1.0 - sga) * ts[0] + 0.25 * (1.0 + sga) * ((1.0 - tga) * ts[1] + (1.0 + tga) * ts[2]);
        QPoint<double> q;
        map_point(e, sgg, tgg, x, 1.0, q);
        cplx<double> bcv = cmk(0.0, 0.0);
        for (int a = 0; a < nv; ++a) bcv += bc[a] * q.sh[a];
        o.rhs = ((o.v.H * P.tao + o.v.E * beta) * bcv) * -1.0;
    }
    return o;
}

// FP32 form of warp_singular's G, H, H^T and E (no right-hand-side terms)
// for the mixed-precision assembly.  p holds the element's vertices minus
// the collocation point (differences taken in FP64, then rounded), so no
// large coordinate enters the float arithmetic.  The rule subtracts no
// static part anywhere (Stokes contour form for E, Duffy-collapsed
// sub-triangles for G, H, H^T), so FP32 keeps about 1e-6 relative accuracy
// on the self entry, below the complex64 storage of A it is added to.  The
// FP64 rule made the near-pair kernel FP64-pipe bound on GB300.
__device__ __forceinline__ KVals<float> warp_singular_f(int nv, const float p[4][3], const float nx[3], float k,
                                                        float wr) {
    const int lane = threadIdx.x & 31;
    const float wnu2 = k * k;
    const float i4pi = (float)(1.0 / kPI4);
    cplx<float> zG = {0.f, 0.f}, zH = zG, zHT = zG, zE = zG;
    const int n_edge = nv * 12, n_area = nv * 32;
    for (int f = lane; f < n_edge + n_area; f += 32) {
        if (f < n_edge) {
            // contour term of E: 4 sections x 3-point Gauss per edge
            const int ieg = f / 12, rem = f - ieg * 12, isec = rem / 3, ig = rem - isec * 3;
            const int ig1 = ieg + 1 == nv ? 0 : ieg + 1;
            float dif[3], len2 = 0.f;
#pragma unroll
            for (int c = 0; c < 3; ++c) { dif[c] = p[ig1][c] - p[ieg][c]; len2 = fmaf(dif[c], dif[c], len2); }
            const float len = sqrtf(len2), il = 1.f / len;
            const float sga = (-0.75f + 0.5f * (float)isec) + 0.25f * c_glxf[3][ig];
            const float wga = c_glwf[3][ig] * (0.125f * len);
            float d[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) d[c] = fmaf(dif[c], 0.5f * (sga + 1.f), p[ieg][c]);
            const float r = sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]), ir = 1.f / r;
            float sn, cs;
            phase_sincos(wr * r, &sn, &cs);
            // grad G = G (-1/r + i wr) r^, crossed with the edge direction
            const cplx<float> zg = cplx<float>{cs * i4pi * ir, sn * i4pi * ir} * cplx<float>{-ir, wr};
            const float t0 = (d[1] * dif[2] - d[2] * dif[1]) * ir * il;
            const float t1 = (d[2] * dif[0] - d[0] * dif[2]) * ir * il;
            const float t2 = (d[0] * dif[1] - d[1] * dif[0]) * ir * il;
            zE += zg * ((t0 * nx[0] + t1 * nx[1] + t2 * nx[2]) * wga);
        } else {
            // G, H, H^T and the k^2 part of E: 2 sub-triangles per edge from
            // the centre, 4 x 4 Gauss collapsed at the centre (weight 1 + s)
            const int fa = f - n_edge;
            const int ieg = fa / 32, rem = fa - ieg * 32, isec = rem / 16, g = rem - isec * 16;
            const int ig1 = ieg + 1 == nv ? 0 : ieg + 1, ig2 = ieg + nv;
            float ss[3], ts[3], aresub;
            if (nv == 3) {
                aresub = 1.f / 48.f;
                ss[0] = ts[0] = 1.f / 3.f;
                if (isec == 0) { ss[1] = c_csi6f[ieg]; ss[2] = c_csi6f[ig2]; ts[1] = c_eta6f[ieg]; ts[2] = c_eta6f[ig2]; }
                else { ss[1] = c_csi6f[ig2]; ss[2] = c_csi6f[ig1]; ts[1] = c_eta6f[ig2]; ts[2] = c_eta6f[ig1]; }
            } else {
                aresub = 0.125f;
                ss[0] = ts[0] = 0.f;
                if (isec == 0) { ss[1] = c_csi8f[ieg]; ss[2] = c_csi8f[ig2]; ts[1] = c_eta8f[ieg]; ts[2] = c_eta8f[ig2]; }
                else { ss[1] = c_csi8f[ig2]; ss[2] = c_csi8f[ig1]; ts[1] = c_eta8f[ig2]; ts[2] = c_eta8f[ig1]; }
            }
            const int gi = g >> 2, gj = g & 3;
            const float sga = c_glxf[4][gi], tga = c_glxf[4][gj];
            const float wq = c_glwf[4][gi] * c_glwf[4][gj] * (1.f + sga) * aresub;
            const float s = 0.5f * (1.f - sga) * ss[0] + 0.25f * (1.f + sga) * ((1.f - tga) * ss[1] + (1.f + tga) * ss[2]);
            const float t = 0.5f * (1.f - sga) * ts[0] + 0.25f * (1.f + sga) * ((1.f - tga) * ts[1] + (1.f + tga) * ts[2]);
            // shape functions and their derivatives (NC_ComputeParameters)
            float sh[4], ds[4], dt[4];
            if (nv == 3) {
                sh[0] = s; sh[1] = t; sh[2] = 1.f - s - t; sh[3] = 0.f;
                ds[0] = 1.f; ds[1] = 0.f; ds[2] = -1.f; ds[3] = 0.f;
                dt[0] = 0.f; dt[1] = 1.f; dt[2] = -1.f; dt[3] = 0.f;
            } else {
                const float s1 = 0.25f * (s + 1.f), s2 = 0.25f * (s - 1.f), t1 = t + 1.f, t2 = t - 1.f;
                sh[0] = s1 * t1; sh[1] = -s2 * t1; sh[2] = s2 * t2; sh[3] = -s1 * t2;
                ds[0] = 0.25f * (t + 1.f); ds[2] = 0.25f * (t - 1.f); ds[1] = -ds[0]; ds[3] = -ds[2];
                dt[0] = 0.25f * (s + 1.f); dt[2] = 0.25f * (s - 1.f); dt[1] = -dt[2]; dt[3] = -dt[0];
            }
            float d[3], dxs[3], dxt[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                d[c] = 0.f; dxs[c] = 0.f; dxt[c] = 0.f;
                for (int a = 0; a < nv; ++a) {
                    d[c] = fmaf(sh[a], p[a][c], d[c]);
                    dxs[c] = fmaf(ds[a], p[a][c], dxs[c]);
                    dxt[c] = fmaf(dt[a], p[a][c], dxt[c]);
                }
            }
            const float n0 = dxs[1] * dxt[2] - dxt[1] * dxs[2];
            const float n1 = dxs[2] * dxt[0] - dxt[2] * dxs[0];
            const float n2 = dxs[0] * dxt[1] - dxt[0] * dxs[1];
            const float jl = sqrtf(n0 * n0 + n1 * n1 + n2 * n2), ijl = 1.f / jl;
            const float ny[3] = {n0 * ijl, n1 * ijl, n2 * ijl};
            const float r = sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]), ir = 1.f / r;
            float sn, cs;
            phase_sincos(wr * r, &sn, &cs);
            const float re2 = wq * jl * i4pi * ir;
            const cplx<float> zg = {cs * re2, sn * re2};
            const cplx<float> zh = zg * cplx<float>{-ir, wr};
            const float re1 = (d[0] * ny[0] + d[1] * ny[1] + d[2] * ny[2]) * ir;
            const float rr2 = -(d[0] * nx[0] + d[1] * nx[1] + d[2] * nx[2]) * ir;
            zG += zg;
            zH += zh * re1;
            zHT += zh * rr2;
            zE += zg * (wnu2 * (nx[0] * ny[0] + nx[1] * ny[1] + nx[2] * ny[2]));
        }
    }
    return {warp_sum(zG), warp_sum(zH), warp_sum(zHT), warp_sum(zE)};
}

}  // namespace bem
