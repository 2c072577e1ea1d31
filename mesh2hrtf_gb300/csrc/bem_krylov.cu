// bem_krylov.cu - dense complex matrix-vector products and the vector kernels
// of the restarted GMRES.
//
// Matrix-vector product (the solve's HBM-bound hot loop, the counterpart of
// NumCalc's NC_MatrixVectorMultiplication case 0, NC_CommonFunctions.cpp:
// 1237-1245): a block of 8 warps owns 16 consecutive rows (2 per warp) and
// walks the columns in tiles of 1024; the tile of x is staged once in shared
// memory for all 16 rows, every lane then streams 16-byte loads of A (two
// complex64 or one complex128 entry) for both of its rows.  Partial sums stay
// in registers and are reduced across the warp in FP64 at the end.
#include <cuda_runtime.h>

#include <atomic>

#include "bem_internal.h"

namespace bem {
namespace {

constexpr int kRowsPerWarp = 2;
constexpr int kWarps = 8;
constexpr int kRowsPerBlock = kRowsPerWarp * kWarps;
constexpr int kTile = 1024;

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// error-free transformations (Knuth two-sum, FMA two-product)
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// FP64: y = r_in - A x or A x
__global__ void __launch_bounds__(256) k_matvec64(const double2 *__restrict__ A, int n, size_t lda,
                                                  const double2 *__restrict__ x,
                                                  const double2 *__restrict__ r_in, double2 *__restrict__ y,
                                                  const int *done) {
    __shared__ double2 xs[kTile];
    if (done && *done) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int row0 = blockIdx.x * kRowsPerBlock + warp * kRowsPerWarp;
    double re[kRowsPerWarp] = {0.0, 0.0}, im[kRowsPerWarp] = {0.0, 0.0};
    for (int base = 0; base < n; base += kTile) {
        const int len = min(kTile, n - base);
        __syncthreads();
        for (int t = threadIdx.x; t < len; t += blockDim.x) xs[t] = x[base + t];
        __syncthreads();
#pragma unroll
        for (int r = 0; r < kRowsPerWarp; ++r) {
            const int row = row0 + r;
            if (row >= n) continue;
            const double2 *Ar = A + (size_t)row * lda + base;
#pragma unroll 4
            for (int c = lane; c < len; c += 32) {
                const double2 a = __ldcs(Ar + c);
                const double2 xv = xs[c];
                re[r] = fma(a.x, xv.x, re[r]);
                re[r] = fma(-a.y, xv.y, re[r]);
                im[r] = fma(a.x, xv.y, im[r]);
                im[r] = fma(a.y, xv.x, im[r]);
            }
        }
    }
#pragma unroll
    for (int r = 0; r < kRowsPerWarp; ++r) {
        const int row = row0 + r;
        const double sr = warp_sum_d(re[r]), si = warp_sum_d(im[r]);
        if (lane == 0 && row < n) {
            double2 o = make_double2(sr, si);
            if (r_in) { o.x = r_in[row].x - sr; o.y = r_in[row].y - si; }
            y[row] = o;
        }
    }
}

// split x (complex128) into x_hi + x_lo (complex64 each)
__global__ void k_split(const double2 *__restrict__ x, float4 *__restrict__ xf, int n, const int *done) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || (done && *done)) return;
    const double2 v = x[i];
    const float hr = (float)v.x, hi = (float)v.y;
    xf[i] = make_float4(hr, hi, (float)(v.x - (double)hr), (float)(v.y - (double)hi));
}

// complex64 A.  EXACT = false: FP32 products on x_hi, per-lane FP32 sums.
// EXACT = true: two-product/two-sum accumulation of A x_hi plus FP32 A x_lo.
template <bool EXACT>
__global__ void __launch_bounds__(256) k_matvec32(const float2 *__restrict__ A, int n, size_t lda, const float4 *__restrict__ xf,
                                                  const double2 *__restrict__ r_in, double2 *__restrict__ y,
                                                  const int *done) {
    __shared__ float4 xs[kTile];
    if (done && *done) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int row0 = blockIdx.x * kRowsPerBlock + warp * kRowsPerWarp;
    float sr[kRowsPerWarp] = {0.f, 0.f}, si[kRowsPerWarp] = {0.f, 0.f};
    float er[kRowsPerWarp] = {0.f, 0.f}, ei[kRowsPerWarp] = {0.f, 0.f};
    for (int base = 0; base < n; base += kTile) {
        const int len = min(kTile, n - base);
        __syncthreads();
        for (int t = threadIdx.x; t < len; t += blockDim.x) xs[t] = xf[base + t];
        __syncthreads();
#pragma unroll
        for (int r = 0; r < kRowsPerWarp; ++r) {
            const int row = row0 + r;
            if (row >= n) continue;
            const float2 *Ar = A + (size_t)row * lda + base;
            // pairs of entries per 16-byte load where alignment allows
            const bool vec = ((((size_t)row * lda + base) & 1) == 0);
            if (vec) {
                const float4 *A4 = reinterpret_cast<const float4 *>(Ar);
                const int len2 = len >> 1;
#pragma unroll 4
                for (int c = lane; c < len2; c += 32) {
                    const float4 a = __ldcs(A4 + c);
                    const float4 x0 = xs[2 * c], x1 = xs[2 * c + 1];
                    if (!EXACT) {
                        sr[r] = fmaf(a.x, x0.x, sr[r]); sr[r] = fmaf(-a.y, x0.y, sr[r]);
                        si[r] = fmaf(a.x, x0.y, si[r]); si[r] = fmaf(a.y, x0.x, si[r]);
                        sr[r] = fmaf(a.z, x1.x, sr[r]); sr[r] = fmaf(-a.w, x1.y, sr[r]);
                        si[r] = fmaf(a.z, x1.y, si[r]); si[r] = fmaf(a.w, x1.x, si[r]);
                    } else {
                        float p, q, s, e;
                        // entry 0
                        p = a.x * x0.x; q = fmaf(a.x, x0.x, -p); two_sum(sr[r], p, s, e); sr[r] = s; er[r] += e + q;
                        p = -a.y * x0.y; q = fmaf(-a.y, x0.y, -p); two_sum(sr[r], p, s, e); sr[r] = s; er[r] += e + q;
                        p = a.x * x0.y; q = fmaf(a.x, x0.y, -p); two_sum(si[r], p, s, e); si[r] = s; ei[r] += e + q;
                        p = a.y * x0.x; q = fmaf(a.y, x0.x, -p); two_sum(si[r], p, s, e); si[r] = s; ei[r] += e + q;
                        er[r] = fmaf(a.x, x0.z, er[r]); er[r] = fmaf(-a.y, x0.w, er[r]);
                        ei[r] = fmaf(a.x, x0.w, ei[r]); ei[r] = fmaf(a.y, x0.z, ei[r]);
                        // entry 1
                        p = a.z * x1.x; q = fmaf(a.z, x1.x, -p); two_sum(sr[r], p, s, e); sr[r] = s; er[r] += e + q;
                        p = -a.w * x1.y; q = fmaf(-a.w, x1.y, -p); two_sum(sr[r], p, s, e); sr[r] = s; er[r] += e + q;
                        p = a.z * x1.y; q = fmaf(a.z, x1.y, -p); two_sum(si[r], p, s, e); si[r] = s; ei[r] += e + q;
                        p = a.w * x1.x; q = fmaf(a.w, x1.x, -p); two_sum(si[r], p, s, e); si[r] = s; ei[r] += e + q;
                        er[r] = fmaf(a.z, x1.z, er[r]); er[r] = fmaf(-a.w, x1.w, er[r]);
                        ei[r] = fmaf(a.z, x1.w, ei[r]); ei[r] = fmaf(a.w, x1.z, ei[r]);
                    }
                }
                if ((len & 1) && lane == 0) {
                    const int c = len - 1;
                    const float2 a = Ar[c];
                    const float4 x0 = xs[c];
                    sr[r] = fmaf(a.x, x0.x, sr[r]); sr[r] = fmaf(-a.y, x0.y, sr[r]);
                    si[r] = fmaf(a.x, x0.y, si[r]); si[r] = fmaf(a.y, x0.x, si[r]);
                    if (EXACT) {
                        er[r] = fmaf(a.x, x0.z, er[r]); er[r] = fmaf(-a.y, x0.w, er[r]);
                        ei[r] = fmaf(a.x, x0.w, ei[r]); ei[r] = fmaf(a.y, x0.z, ei[r]);
                    }
                }
            } else {
                for (int c = lane; c < len; c += 32) {
                    const float2 a = __ldcs(Ar + c);
                    const float4 x0 = xs[c];
                    sr[r] = fmaf(a.x, x0.x, sr[r]); sr[r] = fmaf(-a.y, x0.y, sr[r]);
                    si[r] = fmaf(a.x, x0.y, si[r]); si[r] = fmaf(a.y, x0.x, si[r]);
                    if (EXACT) {
                        er[r] = fmaf(a.x, x0.z, er[r]); er[r] = fmaf(-a.y, x0.w, er[r]);
                        ei[r] = fmaf(a.x, x0.w, ei[r]); ei[r] = fmaf(a.y, x0.z, ei[r]);
                    }
                }
            }
        }
    }
#pragma unroll
    for (int r = 0; r < kRowsPerWarp; ++r) {
        const int row = row0 + r;
        const double tr = warp_sum_d((double)sr[r] + (double)er[r]);
        const double ti = warp_sum_d((double)si[r] + (double)ei[r]);
        if (lane == 0 && row < n) {
            double2 o = make_double2(tr, ti);
            if (r_in) { o.x = r_in[row].x - tr; o.y = r_in[row].y - ti; }
            y[row] = o;
        }
    }
}

// ---- inner products: partial sums per chunk of rows, then a final pass
// h[l] = sum_i conj(V_l[i]) w[i] for l < nv.  Grid (row chunks, groups of
// kDotVec vectors): a block owns kDotChunk rows (one per thread) for kDotVec
// vectors and writes one partial sum per vector: partial[l * nblk + b].
constexpr int kDotChunk = 256;
constexpr int kDotVec = 8;

__global__ void __launch_bounds__(kDotChunk) k_dot_partial(const double2 *__restrict__ V, size_t ldv, int nv,
                                                           const double2 *__restrict__ w, int n,
                                                           double2 *__restrict__ partial, const int *done) {
    __shared__ double red[kDotChunk / 32][2 * kDotVec];
    if (done && *done) return;
    const int b = blockIdx.x, nblk = gridDim.x, l0 = blockIdx.y * kDotVec;
    const int i = b * kDotChunk + threadIdx.x;
    const double2 wv = i < n ? w[i] : make_double2(0.0, 0.0);
    double acc[2 * kDotVec];
#pragma unroll
    for (int q = 0; q < kDotVec; ++q) {
        double re = 0.0, im = 0.0;
        if (i < n && l0 + q < nv) {
            const double2 a = V[(size_t)(l0 + q) * ldv + i];
            re = fma(a.x, wv.x, a.y * wv.y);
            im = fma(a.x, wv.y, -a.y * wv.x);
        }
        acc[2 * q] = warp_sum_d(re);
        acc[2 * q + 1] = warp_sum_d(im);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < 2 * kDotVec; ++q) red[wid][q] = acc[q];
    __syncthreads();
    if (threadIdx.x < 2 * kDotVec) {
        double t = 0.0;
#pragma unroll
        for (int ww = 0; ww < kDotChunk / 32; ++ww) t += red[ww][threadIdx.x];
        const int q = threadIdx.x >> 1;
        if (l0 + q < nv) {
            double *dst = reinterpret_cast<double *>(partial + (size_t)(l0 + q) * nblk + b);
            dst[threadIdx.x & 1] = t;
        }
    }
}

// h[l] = sum_b partial[l][b]; optionally hsum[l] += h[l]; warp l per vector
__global__ void k_dot_final(const double2 *__restrict__ partial, int nblk, int nv, double2 *__restrict__ h,
                            double2 *__restrict__ hsum, const int *done) {
    if (done && *done) return;
    const int l = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (l >= nv) return;
    double re = 0.0, im = 0.0;
    for (int b = lane; b < nblk; b += 32) {
        const double2 p = partial[(size_t)l * nblk + b];
        re += p.x;
        im += p.y;
    }
    re = warp_sum_d(re);
    im = warp_sum_d(im);
    if (lane == 0) {
        h[l] = make_double2(re, im);
        if (hsum) { hsum[l].x += re; hsum[l].y += im; }
    }
}

// w -= sum_l h[l] V_l
__global__ void k_multi_axpy(const double2 *__restrict__ V, size_t ldv, int nv, const double2 *__restrict__ h,
                             double2 *__restrict__ w, int n, const int *done) {
    extern __shared__ double2 hs[];
    if (done && *done) return;
    for (int l = threadIdx.x; l < nv; l += blockDim.x) hs[l] = h[l];
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double2 acc = w[i];
    for (int l = 0; l < nv; ++l) {
        const double2 v = V[(size_t)l * ldv + i], c = hs[l];
        acc.x -= c.x * v.x - c.y * v.y;
        acc.y -= c.x * v.y + c.y * v.x;
    }
    w[i] = acc;
}

__global__ void __launch_bounds__(512) k_norm2(const double2 *__restrict__ w, int n, double *out) {
    __shared__ double s[16];
    double a = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double2 v = w[i];
        a = fma(v.x, v.x, a);
        a = fma(v.y, v.y, a);
    }
    a = warp_sum_d(a);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) s[wid] = a;
    __syncthreads();
    if (wid == 0) {
        a = lane < (int)(blockDim.x >> 5) ? s[lane] : 0.0;
        a = warp_sum_d(a);
        if (lane == 0) out[0] = a;
    }
}

// v = w / sqrt(nrm2.re) where nrm2 is the complex <w, w>
__global__ void k_scale_inv(const double2 *__restrict__ w, const double *nrm2, double2 *__restrict__ v, int n,
                            const int *done) {
    if (done && *done) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double s = 1.0 / sqrt(nrm2[0]);
    const double2 a = w[i];
    v[i] = make_double2(a.x * s, a.y * s);
}

// One Arnoldi step's Givens work on the device (one thread): column k of H
// from hsum[0..k] and |w|^2, previous rotations, the new rotation, the
// residual estimate |g[k+1]|; sets ctrl->done when it is below the target.
// Clears hsum for the next step.
__global__ void k_givens(int k, int m, double2 *__restrict__ hsum, const double *__restrict__ wnorm2,
                         double2 *__restrict__ H, double2 *__restrict__ cs, double2 *__restrict__ sn,
                         double2 *__restrict__ g, GmresCtrl *ctrl) {
    if (threadIdx.x != 0 || ctrl->done) return;
    for (int l = 0; l <= k; ++l) {
        H[(size_t)l * m + k] = hsum[l];
        hsum[l] = make_double2(0.0, 0.0);
    }
    const double hn = sqrt(wnorm2[0]);
    // previous rotations: [a; b] <- [[conj(c), conj(s)], [-s, c]] [a; b]
    for (int l = 0; l < k; ++l) {
        const double2 a = H[(size_t)l * m + k], b = H[(size_t)(l + 1) * m + k];
        const double2 c = cs[l], s = sn[l];
        H[(size_t)l * m + k] = make_double2(c.x * a.x + c.y * a.y + s.x * b.x + s.y * b.y,
                                            c.x * a.y - c.y * a.x + s.x * b.y - s.y * b.x);
        H[(size_t)(l + 1) * m + k] = make_double2(-(s.x * a.x - s.y * a.y) + c.x * b.x - c.y * b.y,
                                                  -(s.x * a.y + s.y * a.x) + c.x * b.y + c.y * b.x);
    }
    const double2 a = H[(size_t)k * m + k];
    const double den = sqrt(a.x * a.x + a.y * a.y + hn * hn);
    double2 c, s;
    if (den == 0.0) { c = make_double2(1.0, 0.0); s = make_double2(0.0, 0.0); }
    else { c = make_double2(a.x / den, a.y / den); s = make_double2(hn / den, 0.0); }
    cs[k] = c;
    sn[k] = s;
    H[(size_t)k * m + k] = make_double2(c.x * a.x + c.y * a.y + s.x * hn, c.x * a.y - c.y * a.x + s.y * hn);
    const double2 gk = g[k];
    g[k + 1] = make_double2(-(s.x * gk.x - s.y * gk.y), -(s.x * gk.y + s.y * gk.x));
    g[k] = make_double2(c.x * gk.x + c.y * gk.y, c.x * gk.y - c.y * gk.x);
    const double res = sqrt(g[k + 1].x * g[k + 1].x + g[k + 1].y * g[k + 1].y);
    ctrl->kdone = k + 1;
    ctrl->res = res;
    if (!(res > ctrl->thr) || hn == 0.0 || !isfinite(res)) ctrl->done = 1;
}

__global__ void k_axpy(const double2 *__restrict__ z, double2 *__restrict__ x, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double2 a = z[i];
    double2 b = x[i];
    b.x += a.x;
    b.y += a.y;
    x[i] = b;
}

__global__ void k_update_x(const double2 *__restrict__ V, int ldv, int nv, const double2 *__restrict__ y,
                           double2 *__restrict__ x, int n) {
    extern __shared__ double2 ys[];
    for (int l = threadIdx.x; l < nv; l += blockDim.x) ys[l] = y[l];
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double2 acc = x[i];
    for (int l = 0; l < nv; ++l) {
        const double2 v = V[(size_t)l * ldv + i], c = ys[l];
        acc.x += c.x * v.x - c.y * v.y;
        acc.y += c.x * v.y + c.y * v.x;
    }
    x[i] = acc;
}

std::atomic<long long> g_launches{0};

}  // namespace

void count_launches(int k) { g_launches.fetch_add(k, std::memory_order_relaxed); }
long long launches() { return g_launches.load(std::memory_order_relaxed); }

cudaError_t launch_matvec(int prec, bool exact, const void *A, int n, size_t lda, const double *x,
                          const double *r_in, double *y, void *xf, cudaStream_t st, const int *done) {
    const int grid = (n + kRowsPerBlock - 1) / kRowsPerBlock;
    count_launches(prec == 0 ? 1 : 2);
    if (prec == 0) {
        k_matvec64<<<grid, 256, 0, st>>>((const double2 *)A, n, lda, (const double2 *)x, (const double2 *)r_in,
                                         (double2 *)y, done);
    } else {
        k_split<<<(n + 255) / 256, 256, 0, st>>>((const double2 *)x, (float4 *)xf, n, done);
        if (exact)
            k_matvec32<true><<<grid, 256, 0, st>>>((const float2 *)A, n, lda, (const float4 *)xf,
                                                   (const double2 *)r_in, (double2 *)y, done);
        else
            k_matvec32<false><<<grid, 256, 0, st>>>((const float2 *)A, n, lda, (const float4 *)xf,
                                                    (const double2 *)r_in, (double2 *)y, done);
    }
    return cudaGetLastError();
}

int dot_blocks(int n) { return (n + kDotChunk - 1) / kDotChunk; }

cudaError_t launch_multi_dot(const double *V, size_t ldv, int nv, const double *w, int n, double *partial,
                             double *h, double *hsum, cudaStream_t st, const int *done) {
    const int nb = dot_blocks(n);
    count_launches(2);
    dim3 grid(nb, (nv + kDotVec - 1) / kDotVec);
    k_dot_partial<<<grid, kDotChunk, 0, st>>>((const double2 *)V, ldv, nv, (const double2 *)w, n, (double2 *)partial,
                                              done);
    k_dot_final<<<(nv + 7) / 8, 256, 0, st>>>((const double2 *)partial, nb, nv, (double2 *)h, (double2 *)hsum, done);
    return cudaGetLastError();
}

cudaError_t launch_multi_axpy(const double *V, size_t ldv, int nv, const double *h, double *w, int n,
                              cudaStream_t st, const int *done) {
    count_launches(1);
    k_multi_axpy<<<(n + 255) / 256, 256, nv * sizeof(double2), st>>>((const double2 *)V, ldv, nv,
                                                                     (const double2 *)h, (double2 *)w, n, done);
    return cudaGetLastError();
}

cudaError_t launch_norm2(const double *w, int n, double *out, cudaStream_t st) {
    count_launches(1);
    k_norm2<<<1, 512, 0, st>>>((const double2 *)w, n, out);
    return cudaGetLastError();
}

cudaError_t launch_scale_inv(const double *w, const double *nrm2, double *v, int n, cudaStream_t st,
                             const int *done) {
    count_launches(1);
    k_scale_inv<<<(n + 255) / 256, 256, 0, st>>>((const double2 *)w, nrm2, (double2 *)v, n, done);
    return cudaGetLastError();
}

cudaError_t launch_givens(int k, int m, double *hsum, const double *wnorm2, double *H, double *cs, double *sn,
                          double *g, GmresCtrl *ctrl, cudaStream_t st) {
    count_launches(1);
    k_givens<<<1, 32, 0, st>>>(k, m, (double2 *)hsum, wnorm2, (double2 *)H, (double2 *)cs, (double2 *)sn,
                               (double2 *)g, ctrl);
    return cudaGetLastError();
}

cudaError_t launch_axpy(const double *z, double *x, int n, cudaStream_t st) {
    count_launches(1);
    k_axpy<<<(n + 255) / 256, 256, 0, st>>>((const double2 *)z, (double2 *)x, n);
    return cudaGetLastError();
}

cudaError_t launch_update_x(const double *V, int ldv, int nv, const double *y, double *x, int n, cudaStream_t st) {
    count_launches(1);
    k_update_x<<<(n + 255) / 256, 256, nv * sizeof(double2), st>>>((const double2 *)V, ldv, nv,
                                                                    (const double2 *)y, (double2 *)x, n);
    return cudaGetLastError();
}

}  // namespace bem
