/* Test infrastructure (oracle only): plain-C FP64 restatement of the
 * reference NumCalc traditional-BEM path.  See bem_oracle.h.  Loop order and
 * floating-point expression order follow the cited reference routines so
 * that, compiled without FMA contraction, results agree with the reference
 * to rounding; the reference itself (oracle/_ref) pins this file in the
 * tests.  Reference paths are relative to mesh2hrtf/NumCalc/src/. */
#include "bem_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define PI4 12.566370614359172944  /* NC_ConstantsVariables.h:66 */
#define EPSY 1.0e-14               /* NC_ConstantsVariables.h:68 */
#define MSBE 220                   /* NC_ConstantsVariables.h:63 */

typedef struct { double re, im; } cx;

static inline cx cmk(double r, double i) { cx z = {r, i}; return z; }
static inline cx cmul(cx a, cx b) { return cmk(a.re * b.re - a.im * b.im, a.im * b.re + a.re * b.im); }
static inline cx cadd(cx a, cx b) { return cmk(a.re + b.re, a.im + b.im); }
static inline cx csub(cx a, cx b) { return cmk(a.re - b.re, a.im - b.im); }
static inline cx cscl(cx a, double s) { return cmk(a.re * s, a.im * s); }
static inline double cabs_(cx a) { return sqrt(a.re * a.re + a.im * a.im); }

/* ---------------------------------------------------------------- tables */
/* Local node coordinates, NC_Arrays.h:126-129. */
static const double CSI8[8] = {1.0, -1.0, -1.0, 1.0, 0.0, -1.0, 0.0, 1.0};
static const double ETA8[8] = {1.0, 1.0, -1.0, -1.0, 1.0, 0.0, -1.0, 0.0};
static const double CSI6[6] = {1.0, 0.0, 0.0, 0.5, 0.0, 0.5};
static const double ETA6[6] = {0.0, 1.0, 0.0, 0.5, 0.5, 0.0};

/* Gauss-Legendre on [-1, 1], 15-decimal published values (the precision
 * the reference tabulates, NC_IntegrationConstants.h:26-49), positive half. */
static const double GL_X[7][3] = {{0}, {0.0}, {0.577350269189626},
    {0.0, 0.774596669241483}, {0.339981043584856, 0.861136311594053},
    {0.0, 0.538469310105683, 0.906179845938664},
    {0.238619186083197, 0.661209386466265, 0.932469514203152}};
static const double GL_W[7][3] = {{0}, {2.0}, {1.0},
    {0.888888888888889, 0.555555555555556}, {0.652145154862546, 0.347854845137454},
    {0.568888888888889, 0.478628670499366, 0.236926885056189},
    {0.467913934572691, 0.360761573048139, 0.171324492379170}};

/* Ascending abscissae as BLGauCooWe lays them out (NC_CommonFunctions.cpp:412-1063). */
static void gauss_line(int n, double *x, double *w)
{
    int h = n / 2;
    if (n % 2) {
        x[h] = GL_X[n][0]; w[h] = GL_W[n][0];
        for (int i = 1; i <= h; ++i) {
            x[h + i] = GL_X[n][i]; x[h - i] = -GL_X[n][i];
            w[h + i] = w[h - i] = GL_W[n][i];
        }
    } else {
        for (int i = 0; i < h; ++i) {
            x[h + i] = GL_X[n][i]; x[h - 1 - i] = -GL_X[n][i];
            w[h + i] = w[h - 1 - i] = GL_W[n][i];
        }
    }
}

/* Triangle rules on the (1,0),(0,1),(0,0) triangle, weights summing to 0.5:
 * centroid rule, Strang-Fix 4-point (degree 3), Radon 7-point (degree 5) and
 * the 13-point degree-7 rule, at the precision the reference tabulates
 * (NC_IntegrationConstants.h:3729-3865). */
static const double TR1[1][3] = {{1.0 / 3.0, 1.0 / 3.0, 0.5}};
static const double TR4[4][3] = {{1.0 / 3.0, 1.0 / 3.0, -27.0 / 96.0}, {0.2, 0.2, 25.0 / 96.0},
                                 {0.6, 0.2, 25.0 / 96.0}, {0.2, 0.6, 25.0 / 96.0}};
static const double TR7[7][3] = {
    {0.1012865073235, 0.1012865073235, 0.1259391805448 / 2.0},
    {0.7974269853531, 0.1012865073235, 0.1259391805448 / 2.0},
    {0.1012865073235, 0.7974269853531, 0.1259391805448 / 2.0},
    {0.4701420641051, 0.0597158717898, 0.1323941527885 / 2.0},
    {0.4701420641051, 0.4701420641051, 0.1323941527885 / 2.0},
    {0.0597158717898, 0.4701420641051, 0.1323941527885 / 2.0},
    {0.3333333333333, 0.3333333333333, 0.225 / 2.0}};
static const double TR13[13][3] = {
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
    {0.3333333333333, 0.3333333333333, -0.1495700444677 / 2.0}};

/* NC_ComputeGausseanPoints, NC_3dFunctions.cpp:455-530. */
static int gauss_points(int nvert, int order, double *s, double *t, double *w)
{
    if (nvert == 3) {
        const double (*tab)[3];
        int n;
        switch (order) {
        case 1: tab = TR1; n = 1; break;
        case 2: tab = TR4; n = 4; break;
        case 3: tab = TR7; n = 7; break;
        default: tab = TR13; n = 13; break;
        }
        for (int i = 0; i < n; ++i) { s[i] = tab[i][0]; t[i] = tab[i][1]; w[i] = tab[i][2]; }
        return n;
    }
    double x[8], wx[8];
    gauss_line(order, x, wx);
    int k = 0;
    for (int i = 0; i < order; ++i)
        for (int j = 0; j < order; ++j) { s[k] = x[i]; t[k] = x[j]; w[k] = wx[i] * wx[j]; ++k; }
    return k;
}

/* ------------------------------------------------------------ element maps */
typedef struct { int nv; double c[4][3]; } elem_t;

static void load_elem(const or_mesh *m, int j, elem_t *e)
{
    e->nv = m->nvert[j];
    for (int a = 0; a < e->nv; ++a)
        for (int k = 0; k < 3; ++k) e->c[a][k] = m->nodes[3 * m->conn[4 * j + a] + k];
}

/* ---------------------------------------------------- symmetry planes */
/* Images per element: 2^(number of planes), NC_Input.cpp:342-343. */
static int n_images(const or_mesh *m)
{
    int c = 0;
    for (int k = 0; k < 3; ++k) if (m->sym[k]) ++c;
    return 1 << c;
}

/* Axis of reflection number kref = 1 .. nref-1: the images are visited in
 * a Gray-code order, one reflection per step (NC_ReflectPointVector,
 * NC_3dFunctions.cpp:190-228). */
static int reflect_dir(const or_mesh *m, int nref, int kref)
{
    static const int nrefdi[8] = {0, 0, 1, 0, 2, 0, 1, 0};
    int nrdir = 0;
    if (nref == 8) {
        nrdir = nrefdi[kref];
    } else if (nref == 4) {
        int i0 = 0;
        for (int i = 0; i < 3; ++i) if (m->sym[i] == 0) { i0 = i + 1; break; }
        nrdir = i0 + nrefdi[kref];
        if (nrdir >= 3) nrdir -= 3;
    } else if (nref == 2) {
        for (int i = 0; i < 3; ++i) if (m->sym[i] != 0) { nrdir = i; break; }
    }
    return nrdir;
}

/* NC_ReflectElement, NC_3dFunctions.cpp:357-452: mirror the element (already
 * holding the previous image) in the plane of step kref, flip the reflection
 * factor and, for velocity data (ibvj0 == 0), the nodal values at an
 * antisymmetric plane, then swap nodes 0/1 (and 2/3) to keep the normal
 * outward. */
static void reflect_elem(const or_mesh *m, int nref, int kref, int ibvj0, int *ireffac, elem_t *e, cx *bc)
{
    const int d = reflect_dir(m, nref, kref);
    if (m->sym[d] < 0) {
        *ireffac = -*ireffac;
        if (ibvj0 == 0)
            for (int a = 0; a < e->nv; ++a) bc[a] = cmk(-bc[a].re, -bc[a].im);
    }
    for (int a = 0; a < e->nv; ++a) e->c[a][d] = 2.0 * m->sym_coord[d] - e->c[a][d];
    for (int p = 0; p < (e->nv == 4 ? 2 : 1); ++p) {
        const int a = 2 * p, b = 2 * p + 1;
        for (int k = 0; k < 3; ++k) { double t = e->c[a][k]; e->c[a][k] = e->c[b][k]; e->c[b][k] = t; }
        cx t = bc[a]; bc[a] = bc[b]; bc[b] = t;
    }
}

/* NC_ReflectPointVector, NC_3dFunctions.cpp:181-242: image of a source
 * point (ifpoi = 1) or of a plane-wave direction (ifpoi = 0). */
static double reflect_point(const or_mesh *m, int nref, int kref, double *v, double reffac, int ifpoi)
{
    const int d = reflect_dir(m, nref, kref);
    if (ifpoi) v[d] = 2.0 * m->sym_coord[d] - v[d];
    else v[d] = -v[d];
    if (m->sym[d] < 0) reffac = -reffac;
    return reffac;
}

/* NC_ComputeGlobalCoordinates, NC_3dFunctions.cpp:95-129. */
static void global_coords(const elem_t *e, double s, double t, double *x, double *sh)
{
    if (e->nv == 3) {
        sh[0] = s; sh[1] = t; sh[2] = 1.0 - s - t;
    } else {
        double s1 = 0.25 * (s + 1.0), s2 = 0.25 * (s - 1.0), t1 = t + 1.0, t2 = t - 1.0;
        sh[0] = s1 * t1; sh[1] = -s2 * t1; sh[2] = s2 * t2; sh[3] = -s1 * t2;
    }
    for (int i = 0; i < 3; ++i) {
        x[i] = 0.0;
        for (int j = 0; j < e->nv; ++j) x[i] += sh[j] * e->c[j][i];
    }
}

/* NC_ComputeUnitVectorOnElement, NC_3dFunctions.cpp:132-178: unit normal, returns Jacobian. */
static double unit_normal(const elem_t *e, double s, double t, double *nrm)
{
    double ds[4], dt[4], dxds[3], dxdt[3];
    if (e->nv == 3) {
        ds[0] = dt[1] = 1.0; ds[1] = dt[0] = 0.0; ds[2] = dt[2] = -1.0;
    } else {
        ds[0] = 0.25 * (t + 1.0); ds[2] = 0.25 * (t - 1.0); ds[1] = -ds[0]; ds[3] = -ds[2];
        dt[0] = 0.25 * (s + 1.0); dt[2] = 0.25 * (s - 1.0); dt[1] = -dt[2]; dt[3] = -dt[0];
    }
    for (int i = 0; i < 3; ++i) {
        dxds[i] = dxdt[i] = 0.0;
        for (int j = 0; j < e->nv; ++j) { dxds[i] += ds[j] * e->c[j][i]; dxdt[i] += dt[j] * e->c[j][i]; }
    }
    nrm[0] = dxds[1] * dxdt[2] - dxdt[1] * dxds[2];
    nrm[1] = dxds[2] * dxdt[0] - dxdt[2] * dxds[0];
    nrm[2] = dxds[0] * dxdt[1] - dxdt[0] * dxds[1];
    double len = sqrt(nrm[0] * nrm[0] + nrm[1] * nrm[1] + nrm[2] * nrm[2]);
    nrm[0] /= len; nrm[1] /= len; nrm[2] /= len;
    return len;
}

/* NC_ComputeParameters, NC_3dFunctions.cpp:533-572. */
static double point_params(const elem_t *e, double s, double t, double *x, double *nrm,
                           double *sh, int with_bc, const cx *bc, cx *bcval)
{
    global_coords(e, s, t, x, sh);
    double jac = unit_normal(e, s, t, nrm);
    *bcval = cmk(0.0, 0.0);
    if (with_bc)
        for (int i = 0; i < e->nv; ++i) *bcval = cadd(*bcval, cscl(bc[i], sh[i]));
    return jac;
}

void or_geometry(const or_mesh *m, double *centers, double *normals, double *areas)
{
    for (int i = 0; i < m->n_elem; ++i) {
        elem_t e;
        load_elem(m, i, &e);
        double s, t, are0, sh[4], nrm[3];
        if (e.nv == 3) { s = t = 1.0 / 3.0; are0 = 0.5; } else { s = t = 0.0; are0 = 4.0; }
        global_coords(&e, s, t, centers + 3 * i, sh);
        double len = unit_normal(&e, s, t, nrm);
        for (int k = 0; k < 3; ++k) normals[15 * i + k] = nrm[k];
        areas[i] = len * are0;
        for (int j = 0; j < e.nv; ++j) {
            double sj = e.nv == 3 ? CSI6[j] : CSI8[j], tj = e.nv == 3 ? ETA6[j] : ETA8[j];
            unit_normal(&e, sj, tj, nrm);
            for (int k = 0; k < 3; ++k) normals[15 * i + 3 * (j + 1) + k] = nrm[k];
        }
    }
}

/* --------------------------------------------------------- subdivision */
static int subelements(const elem_t *e, const double x[3], double arelj, double *xisbp,
                       double *etsbp, double *fasbp, int *ngsbp)
{
    enum { MNSE = 60, NSE = 4 };
    double xisfp[MNSE][4], etsfp[MNSE][4], xisep[MNSE][4], etsep[MNSE][4];
    double xisp[8], etsp[8], sh[4], cp[3];
    const int nv = e->nv;
    int nsbe = -1, nsfl = 1, jr = 0;
    double faclin = 2.0, dxi = 0.0;
    for (int j = 0; j < nv; ++j) {
        xisfp[0][j] = nv == 3 ? CSI6[j] : CSI8[j];
        etsfp[0][j] = nv == 3 ? ETA6[j] : ETA8[j];
    }
    for (;;) {
        int ndie = 0;
        faclin *= 0.5;
        double arels = arelj * faclin * faclin;
        int nsel = nsfl;
        for (int idi = 0; idi < nsel; ++idi)
            for (int j = 0; j < nv; ++j) { xisep[idi][j] = xisfp[idi][j]; etsep[idi][j] = etsfp[idi][j]; }
        for (int idi = 0; idi < nsel; ++idi) {
            double scent = 0.0, tcent = 0.0;
            for (int j = 0; j < nv; ++j) { scent += xisep[idi][j]; tcent += etsep[idi][j]; }
            scent /= (double)nv;
            tcent /= (double)nv;
            global_coords(e, scent, tcent, cp, sh);
            double dist = 0.0;
            for (int i = 0; i < 3; ++i) { double d = cp[i] - x[i]; dist += d * d; }
            dist = sqrt(dist);
            double ratdis = dist / sqrt(arels);
            if (ratdis < 1.3) {
                ++ndie;
                if (ndie > 15) return -1;
                nsfl = ndie * NSE;
                int nsf0 = nsfl - NSE;
                for (int j = 0; j < nv; ++j) {
                    int j1 = j + 1 == nv ? 0 : j + 1;
                    xisp[j] = xisep[idi][j];
                    xisp[j + nv] = (xisep[idi][j] + xisep[idi][j1]) / 2.0;
                    etsp[j] = etsep[idi][j];
                    etsp[j + nv] = (etsep[idi][j] + etsep[idi][j1]) / 2.0;
                }
                for (int j = 0; j < nv; ++j) {
                    int nsu = nsf0 + j, j1 = j + nv, j2 = j1 - 1;
                    if (j2 < nv) j2 += nv;
                    xisfp[nsu][0] = xisp[j]; xisfp[nsu][1] = xisp[j1];
                    etsfp[nsu][0] = etsp[j]; etsfp[nsu][1] = etsp[j1];
                    if (nv == 4) {
                        xisfp[nsu][2] = scent; xisfp[nsu][3] = xisp[j2];
                        etsfp[nsu][2] = tcent; etsfp[nsu][3] = etsp[j2];
                    } else {
                        xisfp[nsu][2] = xisp[j2]; etsfp[nsu][2] = etsp[j2];
                        xisfp[nsf0 + NSE - 1][j] = xisp[j1];
                        etsfp[nsf0 + NSE - 1][j] = etsp[j1];
                    }
                }
            } else {
                ++nsbe;
                if (nsbe >= MSBE) return -1;
                if (nv == 4) {
                    xisbp[nsbe] = (xisep[idi][0] + xisep[idi][1] + xisep[idi][2] + xisep[idi][3]) / 4.0;
                    etsbp[nsbe] = (etsep[idi][0] + etsep[idi][1] + etsep[idi][2] + etsep[idi][3]) / 4.0;
                    fasbp[nsbe] = faclin;
                } else {
                    double xi = (xisep[idi][0] + xisep[idi][1] + xisep[idi][2]) / 3.0;
                    double et = (etsep[idi][0] + etsep[idi][1] + etsep[idi][2]) / 3.0;
                    for (int j = 0; j < nv; ++j) {
                        dxi = xi - xisep[idi][j];
                        double det = et - etsep[idi][j];
                        if (fabs(dxi - det) < 1.0e-8) { jr = j; break; }
                    }
                    xisbp[nsbe] = xisep[idi][jr];
                    etsbp[nsbe] = etsep[idi][jr];
                    fasbp[nsbe] = dxi >= 0.0 ? faclin : -faclin;
                }
                /* Gauss order from the error estimates of NC_Macros.h:44-50 */
                double disfac = 0.5 / ratdis;
                ngsbp[nsbe] = 6;
                for (int o = 2; o <= 6; ++o) {
                    double eg = 32.0, eh = 64.0 * (2.0 * (double)o + 1.0),
                           ee = 128.0 * ((double)o + 1.0) * (2.0 * (double)o + 1.0);
                    for (int q = 0; q < 2 * o + 1; ++q) eg *= disfac;
                    for (int q = 0; q < 2 * o + 2; ++q) eh *= disfac;
                    for (int q = 0; q < 2 * o + 3; ++q) ee *= disfac;
                    if (ee < 0.001 && eh < 0.001 && eg < 0.001) { ngsbp[nsbe] = o; break; }
                }
            }
        }
        if (ndie == 0) break;
    }
    return nsbe + 1;
}

int or_subelements(const or_mesh *m, int j, const double x[3], double area, double *xi,
                   double *eta, double *fac, int *order)
{
    elem_t e;
    load_elem(m, j, &e);
    return subelements(&e, x, area, xi, eta, fac, order);
}

/* ------------------------------------------------------------ integrals */
typedef struct {
    double k, wr;     /* wave number, harmonic time factor * k */
    cx beta;          /* Burton-Miller coupling */
    double gamma, tao;
} consts_t;

/* NC_RegularIntegration, NC_EquationSystem.cpp:1600-1728.  zr[0..4]: G, H, H^T, E, rhs. */
static int regular(const elem_t *e, double area, const double *x, const double *nx,
                   int ifcrhs, int ibvj, const cx *bc, const consts_t *K, cx zr[5])
{
    double xs[MSBE], es[MSBE], fs[MSBE];
    int ng[MSBE];
    for (int i = 0; i < 5; ++i) zr[i] = cmk(0.0, 0.0);
    int nsbe = subelements(e, x, area, xs, es, fs, ng);
    if (nsbe < 0) return -1;
    for (int jsb = 0; jsb < nsbe; ++jsb) {
        double cs[36], ct[36], cw[36];
        double fase = fs[jsb], fase2 = fase * fase;
        int iforie = fabs(fase - 1.0) < EPSY;
        int np = gauss_points(e->nv, ng[jsb], cs, ct, cw);
        for (int g = 0; g < np; ++g) {
            double xio, eto, weih2;
            if (iforie) { xio = cs[g]; eto = ct[g]; weih2 = cw[g]; }
            else { xio = xs[jsb] + cs[g] * fase; eto = es[jsb] + ct[g] * fase; weih2 = cw[g] * fase2; }
            double y[3], ny[3], sh[4];
            cx bcv;
            double jac = point_params(e, xio, eto, y, ny, sh, ifcrhs, bc, &bcv);
            double wga = weih2 * jac;
            double d[3] = {y[0] - x[0], y[1] - x[1], y[2] - x[2]};
            double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            d[0] /= r; d[1] /= r; d[2] /= r;
            double re1 = K->wr * r, re2 = wga / PI4 / r;
            cx zg = cmk(cos(re1) * re2, sin(re1) * re2);
            cx z1 = cmk(-1.0 / r, K->wr);
            cx zhh = cmul(zg, z1), zht = zhh;
            re1 = d[0] * ny[0] + d[1] * ny[1] + d[2] * ny[2];
            re2 = -(d[0] * nx[0] + d[1] * nx[1] + d[2] * nx[2]);
            zhh = cscl(zhh, re1);
            zht = cscl(zht, re2);
            double rq = re1 * re2;
            re1 = nx[0] * ny[0] + nx[1] * ny[1] + nx[2] * ny[2];
            double dq = r * r;
            z1 = cmk((3.0 / dq - K->k * K->k) * rq + re1 / dq, -K->wr / r * (3.0 * rq + re1));
            cx ze = cmul(zg, z1);
            zr[0] = cadd(zr[0], zg);
            zr[1] = cadd(zr[1], zhh);
            zr[2] = cadd(zr[2], zht);
            zr[3] = cadd(zr[3], ze);
            if (ifcrhs) {
                if (ibvj == 0)
                    zr[4] = cadd(zr[4], cmul(cadd(cscl(zg, K->gamma * K->tao), cmul(zht, K->beta)), bcv));
                if (ibvj == 1)
                    zr[4] = csub(zr[4], cmul(cadd(cscl(zhh, K->gamma * K->tao), cmul(ze, K->beta)), bcv));
            }
        }
    }
    return 0;
}

/* NC_SingularIntegration, NC_EquationSystem.cpp:1408-1597. */
static void singular(const elem_t *e, const double *x, const double *nx, int ifcrhs, int ibvj,
                     const cx *bc, const consts_t *K, cx zr[5])
{
    const int nv = e->nv, ngpo1 = 3, nsec1 = 4, nsec2 = 2;
    double cg[3], wg[3], cs[36], ct[36], cw[36];
    double wnu2 = K->k * K->k;
    cx bcv = cmk(0.0, 0.0);
    for (int i = 0; i < 5; ++i) zr[i] = cmk(0.0, 0.0);
    gauss_line(ngpo1, cg, wg);
    for (int ieg = 0; ieg < nv; ++ieg) {
        int ig1 = ieg + 1 == nv ? 0 : ieg + 1, ig2 = ieg + nv;
        double dif[3], dio[3], len = 0.0;
        for (int i = 0; i < 3; ++i) { dif[i] = e->c[ig1][i] - e->c[ieg][i]; len += dif[i] * dif[i]; }
        len = sqrt(len);
        for (int i = 0; i < 3; ++i) dio[i] = dif[i] / len;
        len /= (2.0 * (double)nsec1);
        cx zre = cmk(0.0, 0.0);
        double delsec = 2.0 / (double)nsec1, secmid = -1.0 - delsec / 2.0;
        for (int isec = 0; isec < nsec1; ++isec) {
            secmid += delsec;
            for (int g = 0; g < ngpo1; ++g) {
                double sga = secmid + cg[g] / (double)nsec1, wga = wg[g] * len, d[3];
                for (int i = 0; i < 3; ++i) d[i] = (e->c[ieg][i] + dif[i] * (sga + 1.0) / 2.0) - x[i];
                double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                d[0] /= r; d[1] /= r; d[2] /= r;
                double re1 = K->wr * r, re2 = PI4 * r;
                cx zg = cmk(cos(re1) / re2, sin(re1) / re2);
                zg = cmul(zg, cmk(-1.0 / r, K->wr));
                cx g0 = cscl(zg, d[0]), g1 = cscl(zg, d[1]), g2 = cscl(zg, d[2]);
                cx w0 = csub(cscl(g1, dio[2]), cscl(g2, dio[1]));
                cx w1 = csub(cscl(g2, dio[0]), cscl(g0, dio[2]));
                cx w2 = csub(cscl(g0, dio[1]), cscl(g1, dio[0]));
                cx s = cadd(cadd(cscl(w0, nx[0]), cscl(w1, nx[1])), cscl(w2, nx[2]));
                zre = cadd(zre, cscl(s, wga));
            }
        }
        zr[3] = cadd(zr[3], zre);
        for (int isec = 0; isec < nsec2; ++isec) {
            double ss[3], ts[3], aresub;
            if (nv == 3) {
                aresub = 1.0 / 24.0 / (double)nsec2;
                ss[0] = ts[0] = 1.0 / 3.0;
                if (isec == 0) { ss[1] = CSI6[ieg]; ss[2] = CSI6[ig2]; ts[1] = ETA6[ieg]; ts[2] = ETA6[ig2]; }
                else { ss[1] = CSI6[ig2]; ss[2] = CSI6[ig1]; ts[1] = ETA6[ig2]; ts[2] = ETA6[ig1]; }
            } else {
                aresub = 0.25 / (double)nsec2;
                ss[0] = ts[0] = 0.0;
                if (isec == 0) { ss[1] = CSI8[ieg]; ss[2] = CSI8[ig2]; ts[1] = ETA8[ieg]; ts[2] = ETA8[ig2]; }
                else { ss[1] = CSI8[ig2]; ss[2] = CSI8[ig1]; ts[1] = ETA8[ig2]; ts[2] = ETA8[ig1]; }
            }
            int np = gauss_points(4, 4, cs, ct, cw);
            for (int g = 0; g < np; ++g) {
                double sga = cs[g], tga = ct[g];
                double sgg = 0.5 * (1.0 - sga) * ss[0] + 0.25 * (1.0 + sga) * ((1.0 - tga) * ss[1] + (1.0 + tga) * ss[2]);
                double tgg = 0.5 * (1.0 - sga) * ts[0] + 0.25 * (1.0 + sga) * ((1.0 - tga) * ts[1] + (1.0 + tga) * ts[2]);
                double y[3], ny[3], sh[4];
                double jac = point_params(e, sgg, tgg, y, ny, sh, ifcrhs, bc, &bcv);
                double wga = cw[g] * (1.0 + sga) * aresub * jac;
                double d[3] = {y[0] - x[0], y[1] - x[1], y[2] - x[2]};
                double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                d[0] /= r; d[1] /= r; d[2] /= r;
                double re1 = K->wr * r, re2 = wga / PI4 / r;
                cx zg = cmk(cos(re1) * re2, sin(re1) * re2);
                cx z1 = cmk(-1.0 / r, K->wr);
                cx zhh = cmul(zg, z1), zht = zhh;
                re1 = d[0] * ny[0] + d[1] * ny[1] + d[2] * ny[2];
                re2 = -(d[0] * nx[0] + d[1] * nx[1] + d[2] * nx[2]);
                zhh = cscl(zhh, re1);
                zht = cscl(zht, re2);
                zr[0] = cadd(zr[0], zg);
                zr[1] = cadd(zr[1], zhh);
                zr[2] = cadd(zr[2], zht);
                zr[3] = cadd(zr[3], cscl(zg, wnu2 * (nx[0] * ny[0] + nx[1] * ny[1] + nx[2] * ny[2])));
                if (ifcrhs && ibvj == 0)
                    zr[4] = cadd(zr[4], cmul(cadd(cscl(zg, K->gamma * K->tao), cmul(zht, K->beta)), bcv));
            }
        }
    }
    if (ifcrhs && ibvj == 1) {
        zr[4] = cmul(cadd(cscl(zr[1], K->gamma * K->tao), cmul(zr[3], K->beta)), bcv);
        zr[4] = cscl(zr[4], -1.0);
    }
}

/* The point at which plane waves take their phase: x minus the plane
 * positions on the axes that carry a plane (NC_EquationSystem.cpp:1743-1748,
 * NC_PostProcessing.cpp:794-799). */
static void plane_wave_origin(const or_mesh *m, const double *x, double *xs)
{
    int any = 0;
    for (int k = 0; k < 3; ++k) { xs[k] = x[k]; if (m->sym[k]) any = 1; }
    if (any)
        for (int k = 0; k < 3; ++k) if (m->sym[k] != 0) xs[k] -= m->sym_coord[k];
}

/* NC_IncidentWaveRHS, NC_EquationSystem.cpp:1731-1812, with the images of
 * the waves and sources in the symmetry planes. */
static cx incident_rhs(const or_mesh *m, const or_freq *f, const double *x, const double *nx, const consts_t *K)
{
    const int nref = n_images(m);
    cx zrc = cmk(0.0, 0.0);
    double xs[3];
    plane_wave_origin(m, x, xs);
    for (int i = 0; i < f->n_plane; ++i) {
        double v[3] = {f->pw_dir[3 * i], f->pw_dir[3 * i + 1], f->pw_dir[3 * i + 2]};
        cx zini = cmk(f->pw_amp[2 * i], f->pw_amp[2 * i + 1]);
        double reffac = 1.0;
        for (int kref = 0; kref < nref; ++kref) {
            if (kref > 0) reffac = reflect_point(m, nref, kref, v, reffac, 0);
            double re1 = (v[0] * xs[0] + v[1] * xs[1] + v[2] * xs[2]) * K->wr;
            cx zg = cmul(cmk(cos(re1) * reffac, sin(re1) * reffac), zini);
            double re2 = K->wr * (v[0] * nx[0] + v[1] * nx[1] + v[2] * nx[2]);
            cx zv = cmk(-zg.im * re2, zg.re * re2);
            zrc = csub(zrc, cadd(cscl(zg, K->gamma), cmul(zv, cscl(K->beta, K->tao))));
        }
    }
    for (int i = 0; i < f->n_point; ++i) {
        double s[3] = {f->ps_xyz[3 * i], f->ps_xyz[3 * i + 1], f->ps_xyz[3 * i + 2]};
        cx zini = cmk(f->ps_amp[2 * i], f->ps_amp[2 * i + 1]);
        double reffac = 1.0;
        for (int kref = 0; kref < nref; ++kref) {
            if (kref > 0) reffac = reflect_point(m, nref, kref, s, reffac, 1);
            double d[3] = {x[0] - s[0], x[1] - s[1], x[2] - s[2]};
            double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            d[0] /= r; d[1] /= r; d[2] /= r;
            double re1 = K->wr * r, re2 = reffac / PI4 / r;
            cx zg = cmul(cmk(cos(re1) * re2, sin(re1) * re2), zini);
            re1 = d[0] * nx[0] + d[1] * nx[1] + d[2] * nx[2];
            cx zv = cmul(cmk(-re1 / r, K->wr * re1), zg);
            zrc = csub(zrc, cadd(cscl(zg, K->gamma), cmul(zv, cscl(K->beta, K->tao))));
        }
    }
    return zrc;
}

static void make_consts(const or_freq *f, consts_t *K)
{
    K->k = f->k;
    K->wr = f->htf * f->k;
    K->gamma = 1.0;
    K->tao = f->tao;
    K->beta = f->tao < 0 ? cmk(0.0, 0.0) : cmk(0.0, f->htf / f->k);
}

static void bc_of(const or_mesh *m, int j, cx *bc)
{
    for (int a = 0; a < 4; ++a) bc[a] = cmk(m->bc_val[8 * j + 2 * a], m->bc_val[8 * j + 2 * a + 1]);
}

int or_assemble(const or_mesh *m, const double *centers, const double *normals, const double *areas,
                const or_freq *f, int row0, int row1, double *A, double *rhs, int nthreads)
{
    consts_t K;
    make_consts(f, &K);
    const int n = m->n_elem;
    int err = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1) reduction(| : err)
#endif
    for (int i = row0; i < row1; ++i) {
        double *Arow = A + 2 * (size_t)(i - row0) * n;
        for (int j = 0; j < 2 * n; ++j) Arow[j] = 0.0;
        const double *x = centers + 3 * i, *nx = normals + 15 * i;
        int ibi = m->bc_type[i] == 1 ? 1 : 0, admi = m->bc_type[i] == 2;
        cx bci[4];
        bc_of(m, i, bci);
        cx zbvi = cmk(0.0, 0.0);
        for (int a = 0; a < m->nvert[i]; ++a) zbvi = cadd(zbvi, bci[a]);
        zbvi = cmk(zbvi.re / (double)m->nvert[i], zbvi.im / (double)m->nvert[i]);
        cx admia = admi ? cmk(m->adm[2 * i], m->adm[2 * i + 1]) : cmk(0.0, 0.0);
        /* free terms, NC_EquationSystem.cpp:220-251 */
        cx aii;
        if (ibi == 0) aii = cscl(csub(cmul(admia, K.beta), cmk(K.gamma, 0.0)), 0.5);
        else aii = cscl(K.beta, -(0.5 * K.tao));
        cx z0 = cmk(0.0, 0.0);
        if (ibi == 0) z0 = cadd(z0, cscl(cscl(cmul(zbvi, K.beta), K.tao), 0.5));
        else z0 = cadd(z0, cscl(cscl(zbvi, K.tao), 0.5));
        if (f->n_plane + f->n_point > 0) z0 = cadd(z0, incident_rhs(m, f, x, nx, &K));
        cx ri = z0;
        Arow[2 * i] = aii.re;
        Arow[2 * i + 1] = aii.im;
        const int nref = n_images(m);
        for (int j = 0; j < n && !err; ++j) {
            elem_t e;
            load_elem(m, j, &e);
            int ibj = m->bc_type[j] == 1 ? 1 : 0, admj = m->bc_type[j] == 2;
            cx bcj[4];
            bc_of(m, j, bcj);
            int ifc = 0;
            for (int a = 0; a < e.nv; ++a) if (cabs_(bcj[a]) > EPSY) { ifc = 1; break; }
            /* images of element j, NC_EquationSystem.cpp:277-300 */
            int ireffac = 1;
            for (int kref = 0; kref < nref; ++kref) {
                if (kref > 0) reflect_elem(m, nref, kref, ibj, &ireffac, &e, bcj);
                cx zr[5];
                if (kref == 0 && j == i) singular(&e, x, nx, ifc, ibj, bcj, &K, zr);
                else if (regular(&e, areas[j], x, nx, ifc, ibj, bcj, &K, zr)) { err = 1; break; }
                cx zs;
                if (ibj == 0) {
                    zs = cadd(cscl(zr[1], K.gamma * K.tao), cmul(zr[3], K.beta));
                    if (admj) {
                        cx Y = cmk(m->adm[2 * j], m->adm[2 * j + 1]);
                        zs = cadd(zs, cmul(cadd(cscl(zr[0], K.gamma), cmul(zr[2], cscl(K.beta, K.tao))), Y));
                    }
                } else {
                    zs = csub(cscl(zr[0], -K.gamma * K.tao), cmul(zr[2], K.beta));
                }
                if (ifc) ri = cadd(ri, zr[4]);
                const double reffact = ireffac == -1 ? -1.0 : 1.0;   /* NC_AssembleTBEM:181 */
                Arow[2 * j] += zs.re * reffact;
                Arow[2 * j + 1] += zs.im * reffact;
            }
        }
        rhs[2 * (i - row0)] = ri.re;
        rhs[2 * (i - row0) + 1] = ri.im;
    }
    return err ? -1 : 0;
}

int or_solve_dense(int n, double *A, const double *b, double *x)
{
    cx *M = (cx *)A;
    cx *y = (cx *)malloc(sizeof(cx) * (size_t)n);
    if (!y) return -1;
    for (int i = 0; i < n; ++i) y[i] = cmk(b[2 * i], b[2 * i + 1]);
    for (int c = 0; c < n; ++c) {
        int p = c;
        double best = cabs_(M[(size_t)c * n + c]);
        for (int r = c + 1; r < n; ++r) {
            double v = cabs_(M[(size_t)r * n + c]);
            if (v > best) { best = v; p = r; }
        }
        if (best == 0.0) { free(y); return -1; }
        if (p != c) {
            for (int k = 0; k < n; ++k) {
                cx t = M[(size_t)c * n + k]; M[(size_t)c * n + k] = M[(size_t)p * n + k]; M[(size_t)p * n + k] = t;
            }
            cx t = y[c]; y[c] = y[p]; y[p] = t;
        }
        cx piv = M[(size_t)c * n + c];
        double dd = piv.re * piv.re + piv.im * piv.im;
        cx inv = cmk(piv.re / dd, -piv.im / dd);
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
        for (int r = c + 1; r < n; ++r) {
            cx l = cmul(M[(size_t)r * n + c], inv);
            M[(size_t)r * n + c] = l;
            cx *row = M + (size_t)r * n, *prow = M + (size_t)c * n;
            for (int k = c + 1; k < n; ++k) row[k] = csub(row[k], cmul(l, prow[k]));
            y[r] = csub(y[r], cmul(l, y[c]));
        }
    }
    for (int r = n - 1; r >= 0; --r) {
        cx s = y[r];
        for (int k = r + 1; k < n; ++k) s = csub(s, cmul(M[(size_t)r * n + k], y[k]));
        cx piv = M[(size_t)r * n + r];
        double dd = piv.re * piv.re + piv.im * piv.im;
        y[r] = cmk((s.re * piv.re + s.im * piv.im) / dd, (s.im * piv.re - s.re * piv.im) / dd);
    }
    for (int i = 0; i < n; ++i) { x[2 * i] = y[i].re; x[2 * i + 1] = y[i].im; }
    free(y);
    return 0;
}

/* NC_IntegrationTBEM, NC_PostProcessing.cpp:1217-1322. */
static cx project_sub(const elem_t *e, const double *xp, double xice, double etce, int ngse,
                      double fase, cx zpot, int ivi, const cx *vel, const consts_t *K, cx zv[3])
{
    cx zsub = cmk(0.0, 0.0), *zp = &zsub;
    double cs[36], ct[36], cw[36];
    double fase2 = fase * fase;
    int iforie = fabs(fase - 1.0) < EPSY;
    int np = gauss_points(e->nv, ngse, cs, ct, cw);
    for (int g = 0; g < np; ++g) {
        double xio, eto, weih2;
        if (iforie) { xio = cs[g]; eto = ct[g]; weih2 = cw[g]; }
        else { xio = xice + cs[g] * fase; eto = etce + ct[g] * fase; weih2 = cw[g] * fase2; }
        double y[3], ny[3], sh[4];
        cx unused;
        double jac = point_params(e, xio, eto, y, ny, sh, ivi, vel, &unused);
        double d[3] = {y[0] - xp[0], y[1] - xp[1], y[2] - xp[2]};
        double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        d[0] /= r; d[1] /= r; d[2] /= r;
        double rk = r * K->wr, re1 = r * PI4;
        cx zgr = cmk(cos(rk) / re1, sin(rk) / re1);
        cx zgikr = cmul(zgr, cmk(-1.0 / r, K->wr));
        double drdnx = d[0] * ny[0] + d[1] * ny[1] + d[2] * ny[2];
        cx zfac1 = cmul(zgr, cmk(drdnx * (K->k * K->k - 3.0 / r / r), K->wr * 3.0 * drdnx / r));
        cx zfac2 = cmk(zgikr.re / (-r), zgikr.im / (-r));
        cx zdgrdn = cscl(zgikr, drdnx);
        double vjacwe = jac * weih2;
        cx z1 = cscl(zpot, vjacwe);
        *zp = cadd(*zp, cmul(zdgrdn, z1));
        for (int k = 0; k < 3; ++k)
            zv[k] = cadd(zv[k], cmul(cadd(cscl(zfac1, d[k]), cscl(zfac2, ny[k])), z1));
        if (ivi)
            for (int a = 0; a < e->nv; ++a) {
                cx zz = cscl(vel[a], vjacwe * sh[a]);
                *zp = csub(*zp, cmul(zgr, zz));
                for (int k = 0; k < 3; ++k) zv[k] = csub(zv[k], cmul(cscl(zgikr, -d[k]), zz));
            }
    }
    return zsub;
}

int or_project(const or_mesh *m, const double *centers, const double *normals, const double *areas,
               const or_freq *f, const double *phi, const double *vel, int npts, const double *pts,
               double *pot, double *grad, int nthreads)
{
    (void)centers; (void)normals;
    consts_t K;
    make_consts(f, &K);
    int err = 0;
    const int nref = n_images(m);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 4) reduction(| : err)
#endif
    for (int p = 0; p < npts; ++p) {
        const double *xp = pts + 3 * p;
        cx zp_tot = cmk(0.0, 0.0), zv_tot[3] = {{0, 0}, {0, 0}, {0, 0}};
        for (int j = 0; j < m->n_elem && !err; ++j) {
            elem_t e;
            load_elem(m, j, &e);
            cx zpoto = cmk(phi[2 * j], phi[2 * j + 1]), v[4];
            int ivi = 0;
            for (int a = 0; a < e.nv; ++a) {
                v[a] = cmk(vel[8 * j + 2 * a], vel[8 * j + 2 * a + 1]);
                if (cabs_(v[a]) > EPSY) ivi = 1;
            }
            /* images of element j: velocity data (ibvj0 = 0) flips at
             * antisymmetric planes, the potential with the reflection
             * factor (NC_PostProcessing.cpp:925-972) */
            int ireffac = 1;
            for (int kref = 0; kref < nref; ++kref) {
                if (kref > 0) reflect_elem(m, nref, kref, 0, &ireffac, &e, v);
                cx zpot = ireffac == -1 ? cscl(zpoto, -1.0) : zpoto;
                double xs[MSBE], es[MSBE], fs[MSBE];
                int ng[MSBE];
                int nsbe = subelements(&e, xp, areas[j], xs, es, fs, ng);
                if (nsbe < 0) { err = 1; break; }
                cx zp = cmk(0.0, 0.0), zv[3] = {{0, 0}, {0, 0}, {0, 0}};
                for (int s = 0; s < nsbe; ++s)
                    zp = cadd(zp, project_sub(&e, xp, xs[s], es[s], ng[s], fs[s], zpot, ivi, v, &K, zv));
                if (K.tao != 1.0) { zp = cscl(zp, K.tao); for (int k = 0; k < 3; ++k) zv[k] = cscl(zv[k], K.tao); }
                zp_tot = cadd(zp_tot, zp);
                for (int k = 0; k < 3; ++k) zv_tot[k] = cadd(zv_tot[k], zv[k]);
            }
        }
        /* NC_ContributionIncidentWaves, NC_PostProcessing.cpp:776-866 */
        cx zinc = cmk(0.0, 0.0), vinc[3] = {{0, 0}, {0, 0}, {0, 0}};
        double xs0[3];
        plane_wave_origin(m, xp, xs0);
        for (int i = 0; i < f->n_plane; ++i) {
            double d[3] = {f->pw_dir[3 * i], f->pw_dir[3 * i + 1], f->pw_dir[3 * i + 2]};
            cx zini = cmk(f->pw_amp[2 * i], f->pw_amp[2 * i + 1]);
            double reffac = 1.0;
            for (int kref = 0; kref < nref; ++kref) {
                if (kref > 0) reffac = reflect_point(m, nref, kref, d, reffac, 0);
                double re1 = (d[0] * xs0[0] + d[1] * xs0[1] + d[2] * xs0[2]) * K.wr;
                cx zg = cmul(cmk(cos(re1) * reffac, sin(re1) * reffac), zini);
                zinc = cadd(zinc, zg);
                cx zv = cmk(-zg.im * K.wr, zg.re * K.wr);
                for (int k = 0; k < 3; ++k) vinc[k] = cadd(vinc[k], cscl(zv, d[k]));
            }
        }
        for (int i = 0; i < f->n_point; ++i) {
            double s[3] = {f->ps_xyz[3 * i], f->ps_xyz[3 * i + 1], f->ps_xyz[3 * i + 2]};
            cx zini = cmk(f->ps_amp[2 * i], f->ps_amp[2 * i + 1]);
            double reffac = 1.0;
            for (int kref = 0; kref < nref; ++kref) {
                if (kref > 0) reffac = reflect_point(m, nref, kref, s, reffac, 1);
                double d[3] = {xp[0] - s[0], xp[1] - s[1], xp[2] - s[2]};
                double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                d[0] /= r; d[1] /= r; d[2] /= r;
                double re1 = K.wr * r, re2 = reffac / PI4 / r;
                cx zg = cmul(cmk(cos(re1) * re2, sin(re1) * re2), zini);
                zinc = cadd(zinc, zg);
                cx zv = cmul(cmk(-1.0 / r, K.wr), zg);
                for (int k = 0; k < 3; ++k) vinc[k] = cadd(vinc[k], cscl(zv, d[k]));
            }
        }
        if (f->n_plane || f->n_point) {
            zp_tot = cadd(zp_tot, zinc);
            for (int k = 0; k < 3; ++k) zv_tot[k] = cadd(zv_tot[k], vinc[k]);
        }
        pot[2 * p] = zp_tot.re;
        pot[2 * p + 1] = zp_tot.im;
        for (int k = 0; k < 3; ++k) { grad[6 * p + 2 * k] = zv_tot[k].re; grad[6 * p + 2 * k + 1] = zv_tot[k].im; }
    }
    return err ? -1 : 0;
}

/* ------------------------------------------------------- iterative solver */
/* Complex division as the reference's Complex::operator/ does it
 * (NC_TypeDefinition.h). */
static inline cx cdiv(cx a, cx b)
{
    double t = b.re * b.re + b.im * b.im;
    return cmk((a.re * b.re + a.im * b.im) / t, (a.im * b.re - a.re * b.im) / t);
}

/* Unconjugated dot product Vector<Complex>::operator* (NC_TypeDefinition.h:
 * 403-410), summed in index order. */
static cx cdot(int n, const cx *a, const cx *b)
{
    cx d = cmk(0.0, 0.0);
    for (int i = 0; i < n; ++i) d = cadd(d, cmul(a[i], b[i]));
    return d;
}

/* Threshold ILU of the TBEM branch of NC_IncompleteLUDecomposition
 * (NC_CommonFunctions.cpp:1357-1659): L by rows (diagonal last), U by
 * columns (unit diagonal implied).  The reference finds each product term
 * by scanning boolean masks over all m < i; here the same terms are found by
 * merging the sorted index lists, in the same increasing m, so every entry
 * sees the same operations in the same order. */
typedef struct {
    int n;
    int *lp, *lc;   /* L: row pointers, column indices */
    int *up, *ur;   /* U: column pointers, row indices */
    cx *lv, *uv;
} ilu_t;

static void ilu_free(ilu_t *F)
{
    free(F->lp); free(F->lc); free(F->up); free(F->ur); free(F->lv); free(F->uv);
    memset(F, 0, sizeof(*F));
}

/* dot of L row k (columns < i) with U column c (rows < i), merged in
 * increasing index; the running value z is updated term by term */
static cx ilu_merge(const ilu_t *F, int k, int c, int i, cx z)
{
    int a = F->lp[k], ae = F->lp[k + 1], b = F->up[c], be = F->up[c + 1];
    while (a < ae && b < be) {
        int ca = F->lc[a], rb = F->ur[b];
        if (ca >= i || rb >= i) break;
        if (ca == rb) { z = csub(z, cmul(F->lv[a], F->uv[b])); ++a; ++b; }
        else if (ca < rb) ++a;
        else ++b;
    }
    return z;
}

static int find_idx(const int *idx, int lo, int hi, int v)
{
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (idx[mid] < v) lo = mid + 1; else hi = mid;
    }
    return lo;
}

/* Scales the rows of A and b in place (1410-1423) and factors. */
static int ilu_build(int n, cx *A, cx *b, int scan, ilu_t *F)
{
    static const double thresh[4] = {1.2, 1.0, 0.8, 0.6};
    const double tf = thresh[scan < 0 ? 0 : (scan > 3 ? 3 : scan)];
    memset(F, 0, sizeof(*F));
    F->n = n;
    int *rcnt = (int *)calloc((size_t)n + 1, sizeof(int));
    int *ccnt = (int *)calloc((size_t)n + 1, sizeof(int));
    if (!rcnt || !ccnt) { free(rcnt); free(ccnt); return -1; }
    /* row scaling and the pattern ("trues"): |a_ij| > tf or i == j */
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int i = 0; i < n; ++i) {
        cx *row = A + (size_t)i * n;
        double dw1 = 0.0;
        for (int j = 0; j < n; ++j) dw1 += row[j].re * row[j].re + row[j].im * row[j].im;
        double dwk = sqrt((double)n / dw1);
        int c = 0;
        for (int j = 0; j < n; ++j) {
            row[j] = cscl(row[j], dwk);
            if (cabs_(row[j]) > tf || i == j) ++c;
        }
        b[i] = cscl(b[i], dwk);
        rcnt[i] = c;
    }
    /* L: row i's pattern entries with j <= i; U: column c's entries with
     * row < c.  Count, then fill (rows in increasing order per column). */
    F->lp = (int *)malloc(sizeof(int) * ((size_t)n + 1));
    F->up = (int *)malloc(sizeof(int) * ((size_t)n + 1));
    int *lcnt = (int *)calloc((size_t)n, sizeof(int));
    if (!F->lp || !F->up || !lcnt) { free(rcnt); free(ccnt); free(lcnt); ilu_free(F); return -1; }
    for (int i = 0; i < n; ++i) {
        const cx *row = A + (size_t)i * n;
        for (int j = 0; j < n; ++j) {
            if (!(cabs_(row[j]) > tf || i == j)) continue;
            if (j <= i) ++lcnt[i];
            else ++ccnt[j];
        }
    }
    F->lp[0] = F->up[0] = 0;
    for (int i = 0; i < n; ++i) {
        F->lp[i + 1] = F->lp[i] + lcnt[i];
        F->up[i + 1] = F->up[i] + ccnt[i];
    }
    size_t nl = (size_t)F->lp[n], nu = (size_t)F->up[n];
    F->lc = (int *)malloc(sizeof(int) * (nl ? nl : 1));
    F->lv = (cx *)malloc(sizeof(cx) * (nl ? nl : 1));
    F->ur = (int *)malloc(sizeof(int) * (nu ? nu : 1));
    F->uv = (cx *)malloc(sizeof(cx) * (nu ? nu : 1));
    if (!F->lc || !F->lv || !F->ur || !F->uv) { free(rcnt); free(ccnt); free(lcnt); ilu_free(F); return -1; }
    memset(ccnt, 0, sizeof(int) * (size_t)n);
    for (int i = 0; i < n; ++i) {
        const cx *row = A + (size_t)i * n;
        int q = F->lp[i];
        for (int j = 0; j < n; ++j) {
            if (!(cabs_(row[j]) > tf || i == j)) continue;
            if (j <= i) { F->lc[q] = j; F->lv[q] = row[j]; ++q; }
            else { int p = F->up[j] + ccnt[j]++; F->ur[p] = i; F->uv[p] = row[j]; }
        }
    }
    free(rcnt); free(ccnt); free(lcnt);
    /* transposed position lists: per column c the L entries (k, c), k >= c,
     * and per row r the U entries (r, k), k > r, each in increasing k */
    int *ltp = (int *)calloc((size_t)n + 1, sizeof(int)), *utp = (int *)calloc((size_t)n + 1, sizeof(int));
    int *ltq = (int *)malloc(sizeof(int) * (nl ? nl : 1)), *utq = (int *)malloc(sizeof(int) * (nu ? nu : 1));
    if (!ltp || !utp || !ltq || !utq) { free(ltp); free(utp); free(ltq); free(utq); ilu_free(F); return -1; }
    for (size_t q = 0; q < nl; ++q) ++ltp[F->lc[q] + 1];
    for (size_t q = 0; q < nu; ++q) ++utp[F->ur[q] + 1];
    for (int i = 0; i < n; ++i) { ltp[i + 1] += ltp[i]; utp[i + 1] += utp[i]; }
    {
        int *fl = (int *)malloc(sizeof(int) * (size_t)n), *fu = (int *)malloc(sizeof(int) * (size_t)n);
        if (!fl || !fu) { free(fl); free(fu); free(ltp); free(utp); free(ltq); free(utq); ilu_free(F); return -1; }
        memcpy(fl, ltp, sizeof(int) * (size_t)n);
        memcpy(fu, utp, sizeof(int) * (size_t)n);
        for (int k = 0; k < n; ++k)                       /* rows in increasing k */
            for (int q = F->lp[k]; q < F->lp[k + 1]; ++q) ltq[fl[F->lc[q]]++] = q;
        for (int k = 0; k < n; ++k)                       /* columns in increasing k */
            for (int q = F->up[k]; q < F->up[k + 1]; ++q) utq[fu[F->ur[q]]++] = q;
        free(fl); free(fu);
    }
    /* factorization, loop I of 1611-1658: column i of L (rows k >= i of the
     * pattern), then row i of U (columns k > i) divided by L_ii */
    for (int i = 0; i < n; ++i) {
        const int l0 = ltp[i], l1 = ltp[i + 1];
#ifdef _OPENMP
#pragma omp parallel for schedule(static) if (l1 - l0 > 256)
#endif
        for (int t = l0; t < l1; ++t) {
            const int q = ltq[t];
            int k = find_idx(F->lp, 0, n + 1, q + 1) - 1;   /* row of entry q */
            while (F->lp[k + 1] <= q) ++k;
            F->lv[q] = ilu_merge(F, k, i, i, F->lv[q]);
        }
        const cx dia = F->lv[F->lp[i + 1] - 1];
        const int u0 = utp[i], u1 = utp[i + 1];
#ifdef _OPENMP
#pragma omp parallel for schedule(static) if (u1 - u0 > 256)
#endif
        for (int t = u0; t < u1; ++t) {
            const int p = utq[t];
            int k = find_idx(F->up, 0, n + 1, p + 1) - 1;   /* column of entry p */
            while (F->up[k + 1] <= p) ++k;
            cx z = F->uv[p];
            /* L row i (columns < i) with U column k (rows < i) */
            int a = F->lp[i], ae = F->lp[i + 1], bb = F->up[k], be = F->up[k + 1];
            while (a < ae && bb < be) {
                int ca = F->lc[a], rb = F->ur[bb];
                if (ca >= i || rb >= i) break;
                if (ca == rb) { z = csub(z, cmul(F->lv[a], F->uv[bb])); ++a; ++bb; }
                else if (ca < rb) ++a;
                else ++bb;
            }
            F->uv[p] = cdiv(z, dia);
        }
    }
    free(ltp); free(utp); free(ltq); free(utq);
    return 0;
}

/* NC_IncompleteLUForBack (NC_CommonFunctions.cpp:1673-1721): y = (LU)^-1 v. */
static void ilu_apply(const ilu_t *F, const cx *v, cx *y)
{
    const int n = F->n;
    for (int i = 0; i < n; ++i) y[i] = v[i];
    y[0] = cdiv(y[0], F->lv[0]);
    for (int i = 1; i < n; ++i) {
        int k = F->lp[i + 1] - 1;
        for (int j = F->lp[i]; j < k; ++j) y[i] = csub(y[i], cmul(F->lv[j], y[F->lc[j]]));
        y[i] = cdiv(y[i], F->lv[k]);
    }
    for (int i = n - 1; i > 0; --i)
        for (int j = F->up[i]; j < F->up[i + 1]; ++j) y[F->ur[j]] = csub(y[F->ur[j]], cmul(F->uv[j], y[i]));
}

/* y = A (M^-1 v): NC_MatrixVectorMultiplication case 0 (1211-1245); each row
 * summed in column order, rows split over threads. */
static void precond_matvec(int n, const cx *A, int precond, const ilu_t *F, const double *dsc, const cx *v,
                           cx *t, cx *y)
{
    if (precond == 0) ilu_apply(F, v, t);
    else if (precond == 1) for (int i = 0; i < n; ++i) t[i] = cscl(v[i], dsc[i]);
    else for (int i = 0; i < n; ++i) t[i] = v[i];
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int i = 0; i < n; ++i) {
        const cx *row = A + (size_t)i * n;
        cx s = cmk(0.0, 0.0);
        for (int j = 0; j < n; ++j) s = cadd(s, cmul(row[j], t[j]));
        y[i] = s;
    }
}

/* Tfactor_usy / Tfbelim (NC_TypeDefinition.h:543-594): LU without pivoting
 * in place, then the solve; b is overwritten by the solution. */
static void dense_lu_nopivot(int n, cx *A, cx *b)
{
    for (int i = 0; i < n - 1; ++i) {
        const cx dia = A[(size_t)i * n + i];
        const cx *ri = A + (size_t)i * n;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
        for (int j = i + 1; j < n; ++j) {
            cx *rj = A + (size_t)j * n;
            rj[i] = cdiv(rj[i], dia);
            const cx cji = rj[i];
            for (int k = i + 1; k < n; ++k) rj[k] = csub(rj[k], cmul(ri[k], cji));
        }
        for (int k = i + 1; k < n; ++k) A[(size_t)i * n + k] = cdiv(A[(size_t)i * n + k], dia);
    }
    for (int i = 1; i < n; ++i)
        for (int j = 0; j < i; ++j) b[i] = csub(b[i], cmul(A[(size_t)i * n + j], b[j]));
    for (int i = 0; i < n; ++i) b[i] = cdiv(b[i], A[(size_t)i * n + i]);
    for (int i = n - 1; i > 0; --i)
        for (int j = 0; j < i; ++j) b[j] = csub(b[j], cmul(b[i], A[(size_t)j * n + i]));
}

#include <time.h>
static double now_s(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

int or_solve_cgs(int n, double *Ad, double *bd, int precond, int scan, int niter_max, double tol, double *xd,
                 int *iters, double *rel_err, int nthreads, double *stage_s)
{
    cx *A = (cx *)Ad, *b = (cx *)bd, *x = (cx *)xd;
    double t0 = now_s();
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    if (stage_s) stage_s[0] = stage_s[1] = stage_s[2] = 0.0;
    ilu_t F;
    memset(&F, 0, sizeof(F));
    double *dsc = NULL;
    /* preconditioner set-up (1078-1087) */
    if (precond == 0) {
        if (ilu_build(n, A, b, scan, &F) != 0) return -1;
    } else if (precond == 1) {
        /* NC_ComputeScalingVector, 1322-1354 */
        dsc = (double *)malloc(sizeof(double) * (size_t)n);
        if (!dsc) return -1;
        for (int i = 0; i < n; ++i) {
            double dwk = 0.0;
            const cx *row = A + (size_t)i * n;
            for (int j = 0; j < n; ++j) dwk += row[j].re * row[j].re + row[j].im * row[j].im;
            dsc[i] = sqrt((double)n / dwk);
        }
    }
    double t1 = now_s();
    cx *w = (cx *)malloc(sizeof(cx) * (size_t)n * 10);
    if (!w) { ilu_free(&F); free(dsc); return -1; }
    cx *X = w, *R0 = w + n, *R = w + 2 * (size_t)n, *P = w + 3 * (size_t)n, *V = w + 4 * (size_t)n;
    cx *Q = w + 5 * (size_t)n, *U = w + 6 * (size_t)n, *UQ = w + 7 * (size_t)n, *AUQ = w + 8 * (size_t)n;
    cx *T = w + 9 * (size_t)n;
    for (int j = 0; j < n; ++j) X[j] = cmk(0.0, 0.0);
    precond_matvec(n, A, precond, &F, dsc, X, T, V);
    int direct = 0;
    if (precond == 0)   /* ILU nearly singular (1102-1122): TBEM goes to the direct solver */
        for (int i = 0; i < n; ++i) if (cabs_(V[i]) > 1.0e8) { direct = 1; break; }
    double err_ori = 0.0, err_rel = 1.0;
    int j = 0;
    if (!direct) {
        for (int i = 0; i < n; ++i) U[i] = R[i] = P[i] = R0[i] = csub(b[i], V[i]);
        cx zrjr0 = cmk(0.0, 0.0), zrjr1 = cmk(0.0, 0.0);
        for (j = 0; j <= niter_max; ++j) {
            precond_matvec(n, A, precond, &F, dsc, P, T, V);
            zrjr0 = j == 0 ? cdot(n, R, R0) : zrjr1;
            cx zalph = cdiv(zrjr0, cdot(n, V, R0));
            for (int i = 0; i < n; ++i) Q[i] = csub(U[i], cmul(zalph, V[i]));
            for (int i = 0; i < n; ++i) UQ[i] = cadd(U[i], Q[i]);
            precond_matvec(n, A, precond, &F, dsc, UQ, T, AUQ);
            double dwk1 = 0.0;
            for (int i = 0; i < n; ++i) {
                X[i] = cadd(X[i], cmul(zalph, UQ[i]));
                R[i] = csub(R[i], cmul(zalph, AUQ[i]));
                dwk1 += R[i].re * R[i].re + R[i].im * R[i].im;
            }
            if (j == 0) err_ori = sqrt(dwk1);
            else err_rel = sqrt(dwk1) / err_ori;
            if (err_rel < tol || j == niter_max) {
                for (int i = 0; i < n; ++i) b[i] = X[i];
                break;
            }
            zrjr1 = cdot(n, R, R0);
            cx zbet = cdiv(zrjr1, zrjr0);
            for (int i = 0; i < n; ++i) U[i] = cadd(R[i], cmul(zbet, Q[i]));
            for (int i = 0; i < n; ++i) P[i] = cadd(U[i], cmul(zbet, cadd(Q[i], cmul(zbet, P[i]))));
        }
        if (j >= niter_max) direct = 1;   /* 1181-1191 */
    }
    double t2 = now_s();
    if (direct) {
        /* the reference factors the (scaled) matrix and solves for its
         * (scaled) right-hand side */
        dense_lu_nopivot(n, A, b);
        for (int i = 0; i < n; ++i) x[i] = b[i];
    } else if (precond == 0) {
        ilu_apply(&F, b, x);   /* 1194-1199 */
    } else if (precond == 1) {
        for (int i = 0; i < n; ++i) x[i] = cscl(b[i], dsc[i]);
    } else {
        for (int i = 0; i < n; ++i) x[i] = b[i];
    }
    double t3 = now_s();
    if (stage_s) { stage_s[0] = t1 - t0; stage_s[1] = t2 - t1; stage_s[2] = t3 - t2; }
    if (iters) *iters = j;
    if (rel_err) *rel_err = err_rel;
    ilu_free(&F);
    free(dsc);
    free(w);
    return direct ? 1 : 0;
}
