// bem_direct.cu - dense direct solve of the assembled system: LU without
// pivoting in place, then forward and back substitution, as NumCalc does when
// NC.inp asks for Gaussian elimination (ISOLVER 4) or when CGS fails
// (Tfactor_usy / Tfbelim, NC_TypeDefinition.h:543-594, called from
// NC_IterativeSolverCGS, NC_CommonFunctions.cpp:1181-1191).
//
// Blocked right-looking factorisation A = L U (L unit lower, U upper) in the
// matrix's own precision (complex128 for FP64 solvers, complex64 for mixed
// ones), in panels of kPanel columns:
//   k_lu_panel_col  one launch per pivot column: the multipliers of the rows
//                   below the pivot and their update inside the panel
//   k_lu_trsm       U12 = L11^-1 A12, thread per trailing column
//   k_lu_update     A22 -= L21 U12, 64 x 64 output tiles through shared memory
// The substitutions run in FP64 on blocks of kPanel unknowns: a small
// triangular solve of the diagonal block, then one grid-wide update of the
// remaining rows (thread per row).  Like the reference, no pivoting: a zero
// pivot is reported, not worked around.
#include <cuda_runtime.h>

#include "../../include/bem_gb300.h"
#include "bem_solver.h"

namespace {

constexpr int kPanel = 32;
constexpr int kTile = 64;
constexpr int kChunk = 16;

__device__ __forceinline__ double2 ld2(const double2 &v) { return v; }
__device__ __forceinline__ double2 ld2(const float2 &v) { return make_double2(v.x, v.y); }
__device__ __forceinline__ void st2(double2 &d, double2 v) { d = v; }
__device__ __forceinline__ void st2(float2 &d, double2 v) { d = make_float2((float)v.x, (float)v.y); }

template <typename V> struct Acc;
template <> struct Acc<double2> { using T = double; };
template <> struct Acc<float2> { using T = float; };

template <typename V>
__device__ __forceinline__ V cmul(V a, V b) {
    V r;
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.x * b.y + a.y * b.x;
    return r;
}
template <typename V>
__device__ __forceinline__ V csub(V a, V b) {
    V r;
    r.x = a.x - b.x;
    r.y = a.y - b.y;
    return r;
}
// a / b as the reference's Complex::operator/ forms it
template <typename V>
__device__ __forceinline__ V cdiv(V a, V b) {
    const auto t = b.x * b.x + b.y * b.y;
    V r;
    r.x = (a.x * b.x + a.y * b.y) / t;
    r.y = (a.y * b.x - a.x * b.y) / t;
    return r;
}

// multipliers of pivot column i for rows j > i and their update of the
// panel's columns i+1 .. pend-1
template <typename V>
__global__ void __launch_bounds__(256) k_lu_panel_col(V *A, size_t lda, int n, int i, int pend, int *status) {
    const int j = i + 1 + blockIdx.x * blockDim.x + threadIdx.x;
    const V piv = A[(size_t)i * lda + i];
    if (blockIdx.x == 0 && threadIdx.x == 0 && piv.x == 0 && piv.y == 0) atomicExch(status, 1);
    if (j >= n) return;
    V *row = A + (size_t)j * lda;
    const V *prow = A + (size_t)i * lda;
    const V l = cdiv(row[i], piv);
    row[i] = l;
    for (int c = i + 1; c < pend; ++c) row[c] = csub(row[c], cmul(l, prow[c]));
}

// U12 = L11^-1 A12: thread per column c >= k0 + kb
template <typename V>
__global__ void __launch_bounds__(256) k_lu_trsm(V *A, size_t lda, int n, int k0, int kb) {
    __shared__ V L[kPanel][kPanel];
    for (int t = threadIdx.x; t < kb * kb; t += blockDim.x) {
        const int r = t / kb, c = t % kb;
        L[r][c] = A[(size_t)(k0 + r) * lda + k0 + c];
    }
    __syncthreads();
    const int c = k0 + kb + blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    V u[kPanel];
#pragma unroll
    for (int r = 0; r < kPanel; ++r)
        if (r < kb) u[r] = A[(size_t)(k0 + r) * lda + c];
#pragma unroll
    for (int i = 0; i < kPanel; ++i) {
        if (i >= kb) break;
#pragma unroll
        for (int j = i + 1; j < kPanel; ++j)
            if (j < kb) u[j] = csub(u[j], cmul(L[j][i], u[i]));
    }
#pragma unroll
    for (int r = 0; r < kPanel; ++r)
        if (r < kb) A[(size_t)(k0 + r) * lda + c] = u[r];
}

// A22 -= L21 U12 over the trailing block [k1, n) x [k1, n), k1 = k0 + kb;
// 64 x 64 output tiles, 256 threads with 4 x 4 entries each
template <typename V>
__global__ void __launch_bounds__(256) k_lu_update(V *A, size_t lda, int n, int k0, int kb) {
    __shared__ V Ls[kTile][kChunk + 1];
    __shared__ V Us[kChunk][kTile + 1];
    const int k1 = k0 + kb;
    const int j0 = k1 + blockIdx.y * kTile, c0 = k1 + blockIdx.x * kTile;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    V acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b].x = acc[a][b].y = 0;
    for (int kk = 0; kk < kb; kk += kChunk) {
        for (int t = threadIdx.x; t < kTile * kChunk; t += 256) {
            const int r = t / kChunk, q = t % kChunk;
            const int j = j0 + r, col = k0 + kk + q;
            V v;
            v.x = v.y = 0;
            if (j < n && kk + q < kb) v = A[(size_t)j * lda + col];
            Ls[r][q] = v;
        }
        for (int t = threadIdx.x; t < kTile * kChunk; t += 256) {
            const int q = t / kTile, r = t % kTile;
            const int row = k0 + kk + q, c = c0 + r;
            V v;
            v.x = v.y = 0;
            if (c < n && kk + q < kb) v = A[(size_t)row * lda + c];
            Us[q][r] = v;
        }
        __syncthreads();
#pragma unroll 4
        for (int q = 0; q < kChunk; ++q) {
            V lv[4], uv[4];
#pragma unroll
            for (int a = 0; a < 4; ++a) lv[a] = Ls[ty * 4 + a][q];
#pragma unroll
            for (int b = 0; b < 4; ++b) uv[b] = Us[q][tx * 4 + b];
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) {
                    acc[a][b].x += lv[a].x * uv[b].x - lv[a].y * uv[b].y;
                    acc[a][b].y += lv[a].x * uv[b].y + lv[a].y * uv[b].x;
                }
        }
        __syncthreads();
    }
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        const int j = j0 + ty * 4 + a;
        if (j >= n) continue;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int c = c0 + tx * 4 + b;
            if (c < n) A[(size_t)j * lda + c] = csub(A[(size_t)j * lda + c], acc[a][b]);
        }
    }
}

// forward substitution with the unit lower L on the diagonal block [k0, k0+kb)
template <typename V>
__global__ void k_fwd_diag(const V *A, size_t lda, int k0, int kb, double2 *y) {
    if (threadIdx.x != 0) return;
    for (int i = 0; i < kb; ++i) {
        const double2 yi = y[k0 + i];
        for (int j = i + 1; j < kb; ++j) y[k0 + j] = csub(y[k0 + j], cmul(ld2(A[(size_t)(k0 + j) * lda + k0 + i]), yi));
    }
}
// rows j >= k0 + kb: y_j -= L[j][k0 .. k0+kb) y[k0 .. k0+kb)
template <typename V>
__global__ void __launch_bounds__(256) k_fwd_update(const V *A, size_t lda, int n, int k0, int kb, double2 *y) {
    __shared__ double2 ys[kPanel];
    if (threadIdx.x < kb) ys[threadIdx.x] = y[k0 + threadIdx.x];
    __syncthreads();
    const int j = k0 + kb + blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const V *row = A + (size_t)j * lda + k0;
    double2 s = y[j];
    for (int i = 0; i < kb; ++i) s = csub(s, cmul(ld2(row[i]), ys[i]));
    y[j] = s;
}
// back substitution with U on the diagonal block [k0, k0+kb)
template <typename V>
__global__ void k_bwd_diag(const V *A, size_t lda, int k0, int kb, double2 *y) {
    if (threadIdx.x != 0) return;
    for (int i = kb - 1; i >= 0; --i) {
        const double2 xi = cdiv(y[k0 + i], ld2(A[(size_t)(k0 + i) * lda + k0 + i]));
        y[k0 + i] = xi;
        for (int j = 0; j < i; ++j) y[k0 + j] = csub(y[k0 + j], cmul(ld2(A[(size_t)(k0 + j) * lda + k0 + i]), xi));
    }
}
// rows j < k0: y_j -= U[j][k0 .. k0+kb) x[k0 .. k0+kb)
template <typename V>
__global__ void __launch_bounds__(256) k_bwd_update(const V *A, size_t lda, int k0, int kb, double2 *y) {
    __shared__ double2 xs[kPanel];
    if (threadIdx.x < kb) xs[threadIdx.x] = y[k0 + threadIdx.x];
    __syncthreads();
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= k0) return;
    const V *row = A + (size_t)j * lda + k0;
    double2 s = y[j];
    for (int i = 0; i < kb; ++i) s = csub(s, cmul(ld2(row[i]), xs[i]));
    y[j] = s;
}

template <typename V>
cudaError_t factor(V *A, size_t lda, int n, int *status, cudaStream_t st) {
    long long launches = 0;
    for (int k0 = 0; k0 < n; k0 += kPanel) {
        const int kb = min(kPanel, n - k0), pend = k0 + kb;
        for (int i = k0; i < pend; ++i) {
            const int rows = n - i - 1;
            if (rows <= 0) continue;
            k_lu_panel_col<V><<<(rows + 255) / 256, 256, 0, st>>>(A, lda, n, i, pend, status);
            ++launches;
        }
        const int rest = n - pend;
        if (rest > 0) {
            k_lu_trsm<V><<<(rest + 255) / 256, 256, 0, st>>>(A, lda, n, k0, kb);
            const int t = (rest + kTile - 1) / kTile;
            k_lu_update<V><<<dim3(t, t), 256, 0, st>>>(A, lda, n, k0, kb);
            launches += 2;
        }
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    bem::count_launches(launches);
    return cudaSuccess;
}

template <typename V>
cudaError_t substitute(const V *A, size_t lda, int n, double2 *y, cudaStream_t st) {
    long long launches = 0;
    for (int k0 = 0; k0 < n; k0 += kPanel) {
        const int kb = min(kPanel, n - k0), rest = n - k0 - kb;
        k_fwd_diag<V><<<1, 32, 0, st>>>(A, lda, k0, kb, y);
        ++launches;
        if (rest > 0) {
            k_fwd_update<V><<<(rest + 255) / 256, 256, 0, st>>>(A, lda, n, k0, kb, y);
            ++launches;
        }
    }
    for (int k0 = ((n - 1) / kPanel) * kPanel; k0 >= 0; k0 -= kPanel) {
        const int kb = min(kPanel, n - k0);
        k_bwd_diag<V><<<1, 32, 0, st>>>(A, lda, k0, kb, y);
        ++launches;
        if (k0 > 0) {
            k_bwd_update<V><<<(k0 + 255) / 256, 256, 0, st>>>(A, lda, k0, kb, y);
            ++launches;
        }
    }
    bem::count_launches(launches);
    return cudaGetLastError();
}

}  // namespace

extern "C" bem_status bem_solve_direct(bem_solver_t s, bem_solve_info *info) {
    if (!s) return bem::fail(BEM_ERR_INVALID, "null solver");
    if (!s->have_freq) return bem::fail(BEM_ERR_INVALID, "bem_solve_direct before bem_assemble");
    if (s->factored) return bem::fail(BEM_ERR_INVALID, "bem_solve_direct: the matrix is already factored; assemble again");
    if (cudaSetDevice(s->mesh->device) != cudaSuccess) return bem::fail(BEM_ERR_CUDA, "cudaSetDevice failed");
    cudaStream_t st = s->st;
    const int n = s->n;
    BEM_CU(cudaMemsetAsync(s->d.status, 0, sizeof(int), st));
    BEM_CU(cudaEventRecord(s->ev[2], st));
    if (s->prec == BEM_PREC_FP64) BEM_CU(factor((double2 *)s->d.A, s->lda, n, s->d.status, st));
    else BEM_CU(factor((float2 *)s->d.A, s->lda, n, s->d.status, st));
    for (int r = 0; r < s->n_rhs; ++r) {
        const bem::SolverBufs &d = s->buf(r);
        BEM_CU(cudaMemcpyAsync(d.x, d.b, sizeof(double2) * n, cudaMemcpyDeviceToDevice, st));
        if (s->prec == BEM_PREC_FP64) BEM_CU(substitute((const double2 *)s->d.A, s->lda, n, d.x, st));
        else BEM_CU(substitute((const float2 *)s->d.A, s->lda, n, d.x, st));
    }
    BEM_CU(cudaEventRecord(s->ev[3], st));
    int zero_pivot = 0;
    BEM_CU(cudaMemcpyAsync(&zero_pivot, s->d.status, sizeof(int), cudaMemcpyDeviceToHost, st));
    BEM_CU(cudaStreamSynchronize(st));
    float ms = 0.f;
    BEM_CU(cudaEventElapsedTime(&ms, s->ev[2], s->ev[3]));
    s->factored = true;
    s->solved = true;
    s->info.iterations = 0;
    s->info.restarts = 0;
    s->info.rel_residual = 0.0;
    s->info.solve_ms = ms;
    s->info.matvec_ms = 0.0;
    s->info.n_matvec = 0;
    if (info) *info = s->info;
    if (zero_pivot) return bem::fail(BEM_ERR_INVALID, "bem_solve_direct: zero pivot (LU without pivoting)");
    return BEM_OK;
}
