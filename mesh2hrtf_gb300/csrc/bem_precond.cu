// bem_precond.cu - block-Jacobi preconditioner for the GMRES of bem_solve.
//
// The library numbers the unknowns along a Morton (Z-order) curve of the
// element centres, so consecutive unknowns are spatial neighbours and the
// diagonal blocks of A hold the strongest (near-field) couplings.  The
// preconditioner is the block diagonal of A with blocks of kBlock unknowns,
// inverted once per frequency; NumCalc's own preconditioner is a threshold
// ILU on the same near-field entries (NC_CommonFunctions.cpp:1357-1721).
// By default the Krylov kernels apply it with one correction step over
// windows of kPcWin unknowns, M = X (2 I - A_w X) (bem_gmres.cu), which
// needs no further set-up.
//
// Inversion: one CTA per block of any system in the batch, in-place
// Gauss-Jordan with partial pivoting.  complex64 blocks live in shared memory
// (128 KB); complex128 blocks are inverted in a global workspace (L2
// resident).  Inverses are stored transposed so that the application (inside
// the Krylov kernels, bem_gmres.cu) reads them coalesced.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <type_traits>

#include "bem_internal.h"

namespace bem {
namespace {

template <typename T> struct C2;
template <> struct C2<float> { using t = float2; };
template <> struct C2<double> { using t = double2; };

template <typename V> __device__ __forceinline__ V cmul2(V a, V b) {
    V r;
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.x * b.y + a.y * b.x;
    return r;
}
template <typename V> __device__ __forceinline__ V cinv2(V a) {
    // 1/a, scaled to avoid overflow
    auto s = fabs(a.x) > fabs(a.y) ? fabs(a.x) : fabs(a.y);
    decltype(s) ar = a.x / s, ai = a.y / s, d = ar * ar + ai * ai;
    V r;
    r.x = ar / (d * s);
    r.y = -ai / (d * s);
    return r;
}

// In-place Gauss-Jordan on the nb x nb block W (row-major, leading dim ld),
// executed by one CTA.  colk: nb scratch, piv: nb ints.
template <typename T>
__device__ void gauss_jordan(typename C2<T>::t *W, int ld, int nb, typename C2<T>::t *colk, int *piv,
                             int *pivrow, int *singular) {
    using V = typename C2<T>::t;
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int k = 0; k < nb; ++k) {
        // pivot search by warp 0
        if (tid < 32) {
            T best = -1;
            int bi = k;
            for (int i = k + tid; i < nb; i += 32) {
                V a = W[(size_t)i * ld + k];
                T m = a.x * a.x + a.y * a.y;
                if (m > best) { best = m; bi = i; }
            }
            for (int o = 16; o > 0; o >>= 1) {
                T ob = __shfl_down_sync(0xffffffffu, best, o);
                int oi = __shfl_down_sync(0xffffffffu, bi, o);
                if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
            }
            if (tid == 0) {
                *pivrow = bi;
                piv[k] = bi;
                if (!(best > 0)) *singular = 1;
            }
        }
        __syncthreads();
        const int p = *pivrow;
        if (p != k)
            for (int j = tid; j < nb; j += nt) {
                V t = W[(size_t)k * ld + j];
                W[(size_t)k * ld + j] = W[(size_t)p * ld + j];
                W[(size_t)p * ld + j] = t;
            }
        __syncthreads();
        const V inv = cinv2(W[(size_t)k * ld + k]);
        for (int i = tid; i < nb; i += nt) colk[i] = W[(size_t)i * ld + k];
        __syncthreads();
        for (int j = tid; j < nb; j += nt) {
            V a = j == k ? V{1, 0} : W[(size_t)k * ld + j];
            W[(size_t)k * ld + j] = cmul2(a, inv);
        }
        __syncthreads();
        for (int e = tid; e < nb * nb; e += nt) {
            const int i = e / nb, j = e - i * nb;
            if (i == k) continue;
            const V f = colk[i];
            V a = j == k ? V{0, 0} : W[(size_t)i * ld + j];
            const V r = W[(size_t)k * ld + j];
            a.x -= f.x * r.x - f.y * r.y;
            a.y -= f.x * r.y + f.y * r.x;
            W[(size_t)i * ld + j] = a;
        }
        __syncthreads();
    }
    // undo the row interchanges as column interchanges, last first
    for (int k = nb - 1; k >= 0; --k) {
        const int p = piv[k];
        if (p != k)
            for (int i = tid; i < nb; i += nt) {
                V t = W[(size_t)i * ld + k];
                W[(size_t)i * ld + k] = W[(size_t)i * ld + p];
                W[(size_t)i * ld + p] = t;
            }
        __syncthreads();
    }
}

// The same on a full kBlock x kBlock block by NT threads, with compile-time
// indexing and three barriers per pivot: warp 0 finds the pivot (largest
// |a|^2, lowest row on ties) and gathers the pivot column with the rows
// interchanged, the first kBlock threads interchange the rows and scale the
// pivot row, then thread t updates column t % kBlock of rows t / kBlock,
// + NT / kBlock, ...
template <typename T, int NT>
__device__ void gauss_jordan_full(typename C2<T>::t *W, typename C2<T>::t *colk, int *piv, int *pivrow,
                                  int *singular) {
    using V = typename C2<T>::t;
    constexpr int kG = NT / kBlock;
    static_assert(NT % kBlock == 0 && kBlock % 32 == 0, "threads cover whole columns");
    const int tid = threadIdx.x, lane = tid & 31;
    const int j = tid % kBlock, g = tid / kBlock;
    for (int k = 0; k < kBlock; ++k) {
        if (tid < 32) {
            T best = -1;
            int bi = k;
            for (int i = k + lane; i < kBlock; i += 32) {
                const V a = W[i * kBlock + k];
                const T m = a.x * a.x + a.y * a.y;
                if (m > best) { best = m; bi = i; }
            }
            // butterfly: every lane ends with the same (best, bi)
            for (int o = 16; o > 0; o >>= 1) {
                const T ob = __shfl_xor_sync(0xffffffffu, best, o);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
            }
            for (int i = lane; i < kBlock; i += 32) {
                const int src = i == k ? bi : (i == bi ? k : i);
                colk[i] = W[src * kBlock + k];
            }
            if (lane == 0) {
                *pivrow = bi;
                piv[k] = bi;
                if (!(best > 0)) *singular = 1;
            }
        }
        __syncthreads();
        const int p = *pivrow;
        if (tid < kBlock) {
            const V inv = cinv2(colk[k]);
            const V tk = W[k * kBlock + j], tp = W[p * kBlock + j];
            if (p != k) W[p * kBlock + j] = tk;
            const V a = j == k ? V{1, 0} : tp;
            W[k * kBlock + j] = cmul2(a, inv);
        }
        __syncthreads();
        const V r = W[k * kBlock + j];
#pragma unroll 4
        for (int i = g; i < kBlock; i += kG) {
            if (i == k) continue;
            const V f = colk[i];
            V a = j == k ? V{0, 0} : W[i * kBlock + j];
            a.x -= f.x * r.x - f.y * r.y;
            a.y -= f.x * r.y + f.y * r.x;
            W[i * kBlock + j] = a;
        }
        __syncthreads();
    }
    // undo the row interchanges as column interchanges, last first
    for (int k = kBlock - 1; k >= 0; --k) {
        const int p = piv[k];
        if (p != k)
            for (int i = tid; i < kBlock; i += NT) {
                V t = W[i * kBlock + k];
                W[i * kBlock + k] = W[i * kBlock + p];
                W[i * kBlock + p] = t;
            }
        __syncthreads();
    }
}

__device__ __forceinline__ int find_blk(const int *off, int B, int item) {
    int lo = 0, hi = B - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (off[mid] <= item) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// complex64: block in shared memory
constexpr int kBinv32Threads = 1024;
__global__ void __launch_bounds__(kBinv32Threads) k_binv32(const __grid_constant__ PcBatch tb) {
    extern __shared__ float2 smem[];
    __shared__ float2 colk[kBlock];
    __shared__ int piv[kBlock];
    __shared__ int pivrow, singular;
    const int sb = find_blk(tb.off, tb.B, blockIdx.x);
    const PcSys &S = tb.sys[sb];
    const float2 *A = (const float2 *)S.A;
    const size_t lda = S.lda;
    const int b = blockIdx.x - tb.off[sb], r0 = b * kBlock;
    const int nb = min(kBlock, S.n - r0);
    if (threadIdx.x == 0) singular = 0;
    if (nb == kBlock) {
        for (int e = threadIdx.x; e < kBlock * kBlock; e += kBinv32Threads)
            smem[e] = A[(size_t)(r0 + e / kBlock) * lda + r0 + e % kBlock];
        __syncthreads();
        gauss_jordan_full<float, kBinv32Threads>(smem, colk, piv, &pivrow, &singular);
    } else {   // the last, partial block of a system
        for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
            const int i = e / nb, j = e - i * nb;
            smem[i * kBlock + j] = A[(size_t)(r0 + i) * lda + r0 + j];
        }
        __syncthreads();
        gauss_jordan<float>(smem, kBlock, nb, colk, piv, &pivrow, &singular);
    }
    // store transposed: Minv[b][c][r] = inv[r][c]
    float2 *out = (float2 *)S.Minv + (size_t)b * kBlock * kBlock;
    for (int e = threadIdx.x; e < kBlock * kBlock; e += blockDim.x) {
        const int c = e / kBlock, r = e - c * kBlock;
        out[e] = (r < nb && c < nb) ? smem[r * kBlock + c] : make_float2(0.f, 0.f);
    }
    if (threadIdx.x == 0 && singular) atomicMax(S.status, 1);
}

// complex128: block in a global workspace
__global__ void __launch_bounds__(512) k_binv64(const __grid_constant__ PcBatch tb) {
    __shared__ double2 colk[kBlock];
    __shared__ int piv[kBlock];
    __shared__ int pivrow, singular;
    const int sb = find_blk(tb.off, tb.B, blockIdx.x);
    const PcSys &S = tb.sys[sb];
    const double2 *A = (const double2 *)S.A;
    const size_t lda = S.lda;
    const int b = blockIdx.x - tb.off[sb], r0 = b * kBlock;
    const int nb = min(kBlock, S.n - r0);
    double2 *w = (double2 *)S.work + (size_t)b * kBlock * kBlock;
    if (threadIdx.x == 0) singular = 0;
    if (nb == kBlock) {
        for (int e = threadIdx.x; e < kBlock * kBlock; e += 512)
            w[e] = A[(size_t)(r0 + e / kBlock) * lda + r0 + e % kBlock];
        __syncthreads();
        gauss_jordan_full<double, 512>(w, colk, piv, &pivrow, &singular);
    } else {
        for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
            const int i = e / nb, j = e - i * nb;
            w[i * kBlock + j] = A[(size_t)(r0 + i) * lda + r0 + j];
        }
        __syncthreads();
        gauss_jordan<double>(w, kBlock, nb, colk, piv, &pivrow, &singular);
    }
    double2 *out = (double2 *)S.Minv + (size_t)b * kBlock * kBlock;
    for (int e = threadIdx.x; e < kBlock * kBlock; e += blockDim.x) {
        const int c = e / kBlock, r = e - c * kBlock;
        out[e] = (r < nb && c < nb) ? w[r * kBlock + c] : make_double2(0.0, 0.0);
    }
    if (threadIdx.x == 0 && singular) atomicMax(S.status, 1);
}

// fp16 copy of complex64 rows (SplitBatch): one warp per (row, column
// chunk of kMvChunk entries; with a block low-rank copy a block per (block
// row, chunk), only for the segments the copy reads).  The segment's largest component m sets the
// scale 2^(15 - e) with m < 2^e; every component is scaled (exactly) and
// rounded to nearest.  Power-of-two scales keep A16 * rs within one fp16
// rounding of A.  The warp holds its 8 KB segment in registers, so A is
// read once and no block-wide step is needed.
constexpr int kSplitThreads = 256;
constexpr int kSplitWarps = kSplitThreads / 32;

// One row segment (row i, chunk c) by one warp.
__device__ __forceinline__ void split_segment(const SplitSys &S, int i, int c, int lane) {
    const int n = S.n, nch = mv_chunks(n);
    const int c0 = c * kMvChunk, len = min(kMvChunk, n - c0), len2 = len >> 1;
    const float2 *seg = (const float2 *)S.A + (size_t)i * S.lda + c0;   // 8 KB aligned within the row
    const float4 *seg4 = reinterpret_cast<const float4 *>(seg);
    float4 v[kMvChunk / 64];
    float m = 0.f;
#pragma unroll
    for (int q = 0; q < kMvChunk / 64; ++q) {
        const int k = lane + 32 * q;
        v[q] = k < len2 ? __ldcs(seg4 + k) : make_float4(0.f, 0.f, 0.f, 0.f);   // A is streamed
        m = fmaxf(m, fmaxf(fmaxf(fabsf(v[q].x), fabsf(v[q].y)), fmaxf(fabsf(v[q].z), fabsf(v[q].w))));
    }
    float2 last = make_float2(0.f, 0.f);
    if (len & 1) {
        last = seg[len - 1];
        m = fmaxf(m, fmaxf(fabsf(last.x), fabsf(last.y)));
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    int e = 0;
    if (m > 0.f) frexpf(m, &e);   // m = f 2^e, 0.5 <= f < 1
    const float scale = ldexpf(1.f, 15 - e);
    if (lane == 0) S.rs[(size_t)i * nch + c] = ldexpf(1.f, e - 15);
    __half2 *h = (__half2 *)S.A16 + (size_t)i * S.lda + c0;
    uint2 *out = reinterpret_cast<uint2 *>(h);
#pragma unroll
    for (int q = 0; q < kMvChunk / 64; ++q) {
        const int k = lane + 32 * q;
        if (k < len2) {
            const __half2 h0 = __floats2half2_rn(v[q].x * scale, v[q].y * scale);
            const __half2 h1 = __floats2half2_rn(v[q].z * scale, v[q].w * scale);
            out[k] = make_uint2(*reinterpret_cast<const unsigned *>(&h0), *reinterpret_cast<const unsigned *>(&h1));
        }
    }
    if ((len & 1) && lane == 0) h[len - 1] = __floats2half2_rn(last.x * scale, last.y * scale);
}

__global__ void __launch_bounds__(kSplitThreads) k_split16(const __grid_constant__ SplitBatch tb) {
    const int sb = find_blk(tb.off, tb.B, blockIdx.x);
    const SplitSys &S = tb.sys[sb];
    const int n = S.n, nch = mv_chunks(n), lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (S.blr_rank) {
        // block low-rank copy: a block per (block row I, chunk c), converted
        // only for the diagonal chunk (the preconditioner's window) and
        // chunks with a dense block of the block row; warp w takes rows w,
        // w + kSplitWarps, ...
        const int it = blockIdx.x - tb.off[sb], nb = S.blr_nb;
        const int I = it / nch, c = it - (it / nch) * nch;
        if (I >= nb) return;
        bool need = c == I * kBlrB / kMvChunk;
#pragma unroll
        for (int q = 0; q < kMvChunk / kBlrB; ++q) {
            const int J = c * (kMvChunk / kBlrB) + q;
            need |= J < nb && S.blr_rank[(size_t)I * nb + J] < 0;
        }
        if (!need) return;
        for (int r = warp; r < kBlrB; r += kSplitWarps) {
            const int i = I * kBlrB + r;
            if (i < n) split_segment(S, i, c, lane);
        }
        return;
    }
    const long long item = (long long)(blockIdx.x - tb.off[sb]) * kSplitWarps + warp;
    if (item >= (long long)n * nch) return;
    const int i = (int)(item / nch), c = (int)(item - (long long)i * nch);
    split_segment(S, i, c, lane);
}

}  // namespace

void split_batch_finish(SplitBatch &t) {
    t.off[0] = 0;
    for (int b = 0; b < t.B; ++b) {
        const SplitSys &q = t.sys[b];
        t.off[b + 1] = t.off[b] + (q.blr_rank ? q.blr_nb * mv_chunks(q.n)   // a block per (block row, chunk)
                                              : ceil_div((long long)q.n * mv_chunks(q.n), kSplitWarps));
    }
}

cudaError_t launch_split16(const SplitBatch &t, cudaStream_t st) {
    if (t.B <= 0 || t.off[t.B] == 0) return cudaSuccess;
    count_launches(1);
    k_split16<<<t.off[t.B], kSplitThreads, 0, st>>>(t);
    return cudaGetLastError();
}

// NumCalc's scaling preconditioner (NC_ComputeScalingVector,
// NC_CommonFunctions.cpp:1322-1351, TBEM branch): d_i = sqrt(N / sum_j
// |a_ij|^2), applied to the multiplier vector before every product
// (NC_MatrixVectorMultiplication, :1224-1232), i.e. on the right, and to the
// result at the end (:1193-1203).  Here it is the diagonal of M^{-1} in the
// block-Jacobi storage (the caller clears the blocks), so the Krylov kernels
// apply it unchanged.  Warp per row; row sums in the matrix's precision.
template <typename T>
__global__ void __launch_bounds__(256) k_pc_scaling(const PcSys S) {
    using C2 = typename std::conditional<std::is_same<T, double>::value, double2, float2>::type;
    const int lane = threadIdx.x & 31;
    const int i = blockIdx.x * 8 + (threadIdx.x >> 5);
    if (i >= S.n) return;
    const C2 *row = reinterpret_cast<const C2 *>(S.A) + (size_t)i * S.lda;
    T acc = 0;
    for (int j = lane; j < S.n; j += 32) {
        const C2 a = row[j];
        acc += a.x * a.x + a.y * a.y;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane != 0) return;
    if (!(acc > 0)) {
        atomicMax(S.status, 1);
        return;
    }
    const double d = sqrt((double)S.n / (double)acc);
    const int p = i / kBlock, r = i - p * kBlock;
    C2 *M = reinterpret_cast<C2 *>(S.Minv) + (size_t)p * kBlock * kBlock;
    C2 v;
    v.x = (T)d;
    v.y = 0;
    M[(size_t)r * kBlock + r] = v;
}

cudaError_t launch_pc_scaling(const PcSys &s, int prec, cudaStream_t st) {
    if (s.n <= 0) return cudaSuccess;
    const size_t bytes = (size_t)pc_blocks(s.n) * kBlock * kBlock * (prec == 0 ? 16 : 8);
    cudaError_t e = cudaMemsetAsync(s.Minv, 0, bytes, st);
    if (e != cudaSuccess) return e;
    count_launches(1);
    const int grid = (s.n + 7) / 8;
    if (prec == 0) k_pc_scaling<double><<<grid, 256, 0, st>>>(s);
    else k_pc_scaling<float><<<grid, 256, 0, st>>>(s);
    return cudaGetLastError();
}

size_t precond_bytes(int n, int prec) {
    const size_t nb = (size_t)pc_blocks(n);
    const size_t per = (size_t)kBlock * kBlock * (prec == 0 ? 16 : 8);
    return nb * per * (prec == 0 ? 2 : 1);   // FP64 needs the inversion workspace too
}

void pc_batch_finish(PcBatch &t) {
    t.off[0] = 0;
    for (int b = 0; b < t.B; ++b) t.off[b + 1] = t.off[b] + pc_blocks(t.sys[b].n);
}

cudaError_t launch_block_inverse(const PcBatch &t, int prec, cudaStream_t st) {
    if (t.B <= 0 || t.off[t.B] == 0) return cudaSuccess;
    count_launches(1);
    if (prec == 0) {
        k_binv64<<<t.off[t.B], 512, 0, st>>>(t);
    } else {
        const int smem = kBlock * kBlock * sizeof(float2);
        cudaError_t e = cudaFuncSetAttribute(k_binv32, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        k_binv32<<<t.off[t.B], kBinv32Threads, smem, st>>>(t);
    }
    return cudaGetLastError();
}

}  // namespace bem
