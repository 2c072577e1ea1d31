// bem_blr.cu - the block low-rank Krylov copy of a complex64 matrix.
//
// After assembly, every off-diagonal kBlrB x kBlrB block of A (in the
// unknowns' Morton order) is approximated by adaptive cross approximation
// with partial pivoting, in FP32, from A's own entries: take a row's
// residual against the terms so far, pivot on its largest entry, take that
// column's residual and add the rank-one term; the next row is the column
// residual's largest entry among the rows not used yet (k_blr_aca takes two
// such rows per pass, see there).  The approximation stops when the new
// term's Frobenius norm is below kBlrStop times the norm of the sum so far
// (sum of the terms' squared norms).
//
// That stopping rule only looks at the rows and columns it has visited, and
// on blocks of neighbouring element patches it stops early now and then.  So
// a second pass over the whole block checks the result: with kBlrSketch
// Rademacher probes w_p (signs from a hash of the row), sum_p |w_p^T R|^2 /
// kBlrSketch is an unbiased estimate of |R|_F^2 for the residual R = B - U V^T,
// computed as w^T B - (w^T U) V^T.  A block whose estimate is within kBlrTol
// of |B|_F keeps its terms, as fp16 factors with a power-of-two scale per
// term; any other block, and every diagonal block, is read from the fp16
// copy of A, which is made afterwards for those blocks' segments only.  The
// approximation runs one warp per block (lane l holds entries l, l + 32, ...
// of the block's rows and columns), the check one block of 128 threads.
//
// Boundary-element matrices have numerically low-rank off-diagonal blocks
// (the kernels are smooth between separated element patches): on the
// 5120-triangle head-like mesh 60-80 % of the off-diagonal blocks of 256
// unknowns compress to 25-30 terms at 0.5-4 kHz, so the copy holds about
// 1.7 bytes per matrix entry against the fp16 copy's 4.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "bem_internal.h"

namespace bem {
namespace {

constexpr int kBlrWarps = 2;   // small blocks: a slow warp holds few others back

__device__ __forceinline__ float2 cmul2(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float warp_sumf(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
// largest value over the warp and its index (the smaller index on ties)
__device__ __forceinline__ void warp_argmax(float &v, int &idx) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float ov = __shfl_xor_sync(0xffffffffu, v, o);
        const int oi = __shfl_xor_sync(0xffffffffu, idx, o);
        if (ov > v || (ov == v && oi < idx)) {
            v = ov;
            idx = oi;
        }
    }
}
// smallest index over the warp whose row is unused (kBlrB if none)
__device__ __forceinline__ int first_unused(unsigned used, int lane) {
    int cand = kBlrB;
#pragma unroll
    for (int q = 0; q < 8; ++q)
        if (!((used >> q) & 1u)) {
            cand = lane + 32 * q;
            break;
        }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cand = min(cand, __shfl_xor_sync(0xffffffffu, cand, o));
    return cand;
}

// Rademacher probe signs of a row: bit p is the sign of probe p (integer
// hash lowbias32 by C. Wellons)
__device__ __forceinline__ unsigned probe_bits(unsigned x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}
__device__ __forceinline__ float psign(unsigned bits, int p) { return ((bits >> p) & 1u) ? -1.f : 1.f; }

// fp16 pairs of v * 2^(15 - e), e the exponent of the largest component of
// the warp's 256 entries (m = f 2^e, 0.5 <= f < 1); returns e
__device__ __forceinline__ int store_half(const float2 *v, unsigned *out, int lane) {
    float2 a[kBlrB / 32];
    float m = 0.f;
#pragma unroll
    for (int q = 0; q < kBlrB / 32; ++q) {
        a[q] = v[lane + 32 * q];
        m = fmaxf(m, fmaxf(fabsf(a[q].x), fabsf(a[q].y)));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    int e = 0;
    if (m > 0.f) frexpf(m, &e);
    const float sc = ldexpf(1.f, 15 - e);
#pragma unroll
    for (int q = 0; q < kBlrB / 32; ++q) {
        const __half2 h = __floats2half2_rn(a[q].x * sc, a[q].y * sc);
        out[lane + 32 * q] = *reinterpret_cast<const unsigned *>(&h);
    }
    return e;
}

// entry q of a lane's 8 (q = idx >> 5), from lane idx & 31, on every lane
__device__ __forceinline__ float2 pick8(const float2 (&v)[8], int idx) {
    const int sel = idx >> 5;
    float2 p = v[0];
#pragma unroll
    for (int q = 1; q < 8; ++q) {
        p.x = sel == q ? v[q].x : p.x;
        p.y = sel == q ? v[q].y : p.y;
    }
    p.x = __shfl_sync(0xffffffffu, p.x, idx & 31);
    p.y = __shfl_sync(0xffffffffu, p.y, idx & 31);
    return p;
}
// largest |v|^2 over the entries < lim and its index (kBlrB, -1 if none)
__device__ __forceinline__ void argmax8(const float2 (&v)[8], int lim, int lane, float &best, int &idx) {
    best = -1.f;
    idx = kBlrB;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const int j = lane + 32 * q;
        const float a = v[q].x * v[q].x + v[q].y * v[q].y;
        if (j < lim && a > best) {
            best = a;
            idx = j;
        }
    }
    warp_argmax(best, idx);
}
__device__ __forceinline__ unsigned mark_row(unsigned used, int row, int lane) {
    return (row >= 0 && row < kBlrB && lane == (row & 31)) ? used | (1u << (row >> 5)) : used;
}

// Cross approximation with two pivots per pass: rows i1, i2 (the two largest
// entries of the last column residual among unused rows) are taken together,
// so each pass reads the terms so far once for two new terms.  Term 1 pivots
// on row i1's residual; row i2's residual is updated by term 1 and gives
// term 2; the column of term 2 is updated by term 1 likewise.  The result is
// the two-step cross approximation with these pivots; only the choice of i2
// (from the column residual one term earlier) differs from the one-pivot
// method.
__global__ void __launch_bounds__(32 * kBlrWarps) k_blr_aca(const __grid_constant__ BlrBatch tb) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long gb = (long long)blockIdx.x * kBlrWarps + warp;
    if (gb >= tb.off[tb.B]) return;
    int sb = 0;
    while (gb >= tb.off[sb + 1]) ++sb;
    const BlrSys &S = tb.sys[sb];
    const int nb = blr_blocks(S.n);
    const int b = (int)(gb - tb.off[sb]);
    const int I = b / nb, J = b - (b / nb) * nb;
    if (I == J) {
        if (lane == 0) S.rank[b] = -1;
        return;
    }
    const int I0 = I * kBlrB, J0 = J * kBlrB;
    const int m = min(kBlrB, S.n - I0), nc = min(kBlrB, S.n - J0);
    const float2 *A = reinterpret_cast<const float2 *>(S.A);
    const size_t lda = S.lda;
    float2 *U = S.U + (size_t)b * kBlrMaxRank * kBlrB;
    float2 *V = S.V + (size_t)b * kBlrMaxRank * kBlrB;
    unsigned used = 0;   // bit q: row lane + 32 q taken as a pivot row, or past the block
#pragma unroll
    for (int q = 0; q < 8; ++q)
        if (lane + 32 * q >= m) used |= 1u << q;
    const float stop2 = kBlrStop * kBlrStop;
    int i1 = 0, i2 = m > 1 ? 1 : -1, k = 0;
    float norm2 = 0.f;
    bool ok = false;
    for (int pass = 0; pass < kBlrMaxRank + kBlrB && k + 2 <= kBlrMaxRank; ++pass) {
        bool two = i2 >= 0;
        // residuals of rows i1 and i2
        float2 r1[8], r2[8];
        {
            const float2 *a1 = A + (size_t)(I0 + i1) * lda + J0;
            const float2 *a2 = A + (size_t)(I0 + (two ? i2 : i1)) * lda + J0;
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int j = lane + 32 * q;
                r1[q] = j < nc ? a1[j] : make_float2(0.f, 0.f);
                r2[q] = (two && j < nc) ? a2[j] : make_float2(0.f, 0.f);
            }
        }
#pragma unroll 2
        for (int l = 0; l < k; ++l) {
            const float2 u1 = U[(size_t)l * kBlrB + i1];
            const float2 u2 = two ? U[(size_t)l * kBlrB + i2] : make_float2(0.f, 0.f);
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const float2 v = V[(size_t)l * kBlrB + lane + 32 * q];
                const float2 p1 = cmul2(u1, v), p2 = cmul2(u2, v);
                r1[q].x -= p1.x;
                r1[q].y -= p1.y;
                r2[q].x -= p2.x;
                r2[q].y -= p2.y;
            }
        }
        used = mark_row(mark_row(used, i1, lane), i2, lane);
        float best;
        int j1;
        argmax8(r1, nc, lane, best, j1);
        if (!(best > 1e-30f) && two) {
            // row i1 is represented already: row i2 alone gives the term
#pragma unroll
            for (int q = 0; q < 8; ++q) r1[q] = r2[q];
            two = false;
            argmax8(r1, nc, lane, best, j1);
        }
        if (!(best > 1e-30f)) {
            // both rows are represented: the next unused rows
            i1 = first_unused(used, lane);
            if (i1 >= kBlrB) {
                ok = true;
                break;
            }
            i2 = first_unused(mark_row(used, i1, lane), lane);
            if (i2 >= kBlrB) i2 = -1;
            continue;
        }
        // term 1: v1 = r1 / r1[j1]
        {
            const float2 piv = pick8(r1, j1);
            const float pd = 1.f / (piv.x * piv.x + piv.y * piv.y);
            const float2 inv = make_float2(piv.x * pd, -piv.y * pd);
#pragma unroll
            for (int q = 0; q < 8; ++q) r1[q] = lane + 32 * q < nc ? cmul2(r1[q], inv) : make_float2(0.f, 0.f);
        }
        // term 2: row i2's residual after term 1, v2 = r2 / r2[j2]
        int j2 = -1;
        if (two) {
            const float2 c21 = pick8(r2, j1);
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const float2 p = cmul2(c21, r1[q]);
                r2[q].x -= p.x;
                r2[q].y -= p.y;
            }
            argmax8(r2, nc, lane, best, j2);
            if (best > 1e-30f) {
                const float2 piv = pick8(r2, j2);
                const float pd = 1.f / (piv.x * piv.x + piv.y * piv.y);
                const float2 inv = make_float2(piv.x * pd, -piv.y * pd);
#pragma unroll
                for (int q = 0; q < 8; ++q)
                    r2[q] = lane + 32 * q < nc ? cmul2(r2[q], inv) : make_float2(0.f, 0.f);
            } else {
                j2 = -1;
            }
        }
        const bool t2ok = j2 >= 0 && j2 < kBlrB;
        const float2 v1j2 = t2ok ? pick8(r1, j2) : make_float2(0.f, 0.f);
        float nv1 = 0.f, nv2 = 0.f;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int j = lane + 32 * q;
            V[(size_t)k * kBlrB + j] = r1[q];
            nv1 += r1[q].x * r1[q].x + r1[q].y * r1[q].y;
            if (t2ok) {
                V[(size_t)(k + 1) * kBlrB + j] = r2[q];
                nv2 += r2[q].x * r2[q].x + r2[q].y * r2[q].y;
            }
        }
        // residuals of columns j1 and j2
        float2 c1[8], c2[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int i = lane + 32 * q;
            const float2 *arow = A + (size_t)(I0 + min(i, m - 1)) * lda + J0;
            c1[q] = i < m ? arow[j1] : make_float2(0.f, 0.f);
            c2[q] = (t2ok && i < m) ? arow[j2] : make_float2(0.f, 0.f);
        }
        __syncwarp();   // this pass's V rows are in memory for every lane
#pragma unroll 2
        for (int l = 0; l < k; ++l) {
            const float2 w1 = V[(size_t)l * kBlrB + j1];
            const float2 w2 = t2ok ? V[(size_t)l * kBlrB + j2] : make_float2(0.f, 0.f);
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const float2 u = U[(size_t)l * kBlrB + lane + 32 * q];
                const float2 p1 = cmul2(u, w1), p2 = cmul2(u, w2);
                c1[q].x -= p1.x;
                c1[q].y -= p1.y;
                c2[q].x -= p2.x;
                c2[q].y -= p2.y;
            }
        }
        float nu1 = 0.f, nu2 = 0.f;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int i = lane + 32 * q;
            U[(size_t)k * kBlrB + i] = c1[q];
            nu1 += c1[q].x * c1[q].x + c1[q].y * c1[q].y;
            if (t2ok) {
                const float2 p = cmul2(c1[q], v1j2);   // column j2 after term 1
                c2[q].x -= p.x;
                c2[q].y -= p.y;
                U[(size_t)(k + 1) * kBlrB + i] = c2[q];
                nu2 += c2[q].x * c2[q].x + c2[q].y * c2[q].y;
            }
        }
        nu1 = warp_sumf(nu1);
        nv1 = warp_sumf(nv1);
        float tl = nu1 * nv1;
        norm2 += tl;
        k += 1;
        if (t2ok) {
            nu2 = warp_sumf(nu2);
            nv2 = warp_sumf(nv2);
            tl = nu2 * nv2;
            norm2 += tl;
            k += 1;
        }
        __syncwarp();   // this pass's U columns are in memory for every lane
        if (tl <= stop2 * norm2) {
            ok = true;
            break;
        }
        // next rows: the two largest entries of the last column residual
        // among the unused rows
        float la[8];
#pragma unroll
        for (int q = 0; q < 8; ++q)
            la[q] = t2ok ? c2[q].x * c2[q].x + c2[q].y * c2[q].y : c1[q].x * c1[q].x + c1[q].y * c1[q].y;
        float ba = -1.f, bb = -1.f;
        int ia = kBlrB, ib = kBlrB;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const float a = la[q];
            if (!((used >> q) & 1u) && a > ba) {
                ba = a;
                ia = lane + 32 * q;
            }
        }
        warp_argmax(ba, ia);
        if (ia >= kBlrB || ba < 0.f) {
            ok = true;   // every row is a pivot row: the terms reproduce the block
            break;
        }
        const unsigned used2 = mark_row(used, ia, lane);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const float a = la[q];
            if (!((used2 >> q) & 1u) && a > bb) {
                bb = a;
                ib = lane + 32 * q;
            }
        }
        warp_argmax(bb, ib);
        i1 = ia;
        i2 = (ib < kBlrB && bb >= 0.f) ? ib : -1;
    }
    if (lane == 0) S.rank[b] = ok ? k : -1;
}

// The probe check of k_blr_aca's approximations and their fp16 factors;
// blocks it rejects become dense.  One block of 128 threads per matrix block:
// the row's probe signs go to shared memory once, the warps form w_p^T U_l
// (warp w: terms w, w + 4, ...), then thread t streams columns 2t and 2t + 1
// of the block (16-byte loads; the warps together read whole rows),
// accumulating w_p^T B and |B|^2, and subtracts (w_p^T U) V^T.
constexpr int kChkThreads = kBlrB / 2;
constexpr int kChkWarps = kChkThreads / 32;

__global__ void __launch_bounds__(kChkThreads, 6) k_blr_check(const __grid_constant__ BlrBatch tb) {
    __shared__ float2 cw[kBlrSketch][kBlrMaxRank];   // w_p^T U_l
    __shared__ unsigned rbits[kBlrB];                 // probe signs per row
    __shared__ float red[2][kChkWarps];
    __shared__ float tn[kBlrMaxRank];   // term norms
    __shared__ int keep, kept;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const long long gb = blockIdx.x;
    if (gb >= tb.off[tb.B]) return;
    int sb = 0;
    while (gb >= tb.off[sb + 1]) ++sb;
    const BlrSys &S = tb.sys[sb];
    const int nb = blr_blocks(S.n);
    const int b = (int)(gb - tb.off[sb]);
    const int k = S.rank[b];
    if (k < 0) return;
    const int I = b / nb, J = b - (b / nb) * nb;
    const int I0 = I * kBlrB, J0 = J * kBlrB;
    const int m = min(kBlrB, S.n - I0), nc = min(kBlrB, S.n - J0);
    const float2 *A = reinterpret_cast<const float2 *>(S.A);
    const size_t lda = S.lda;
    const float2 *U = S.U + (size_t)b * kBlrMaxRank * kBlrB;
    const float2 *V = S.V + (size_t)b * kBlrMaxRank * kBlrB;
    const unsigned key0 = (unsigned)(gb * kBlrB);
    for (int i = t; i < kBlrB; i += kChkThreads) rbits[i] = probe_bits(key0 + i);
    __syncthreads();
    for (int l = warp; l < k; l += kChkWarps) {
        float pr[kBlrSketch], pi[kBlrSketch];
#pragma unroll
        for (int p = 0; p < kBlrSketch; ++p) pr[p] = pi[p] = 0.f;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const float2 u = U[(size_t)l * kBlrB + lane + 32 * q];   // zero past the block
            const unsigned hb = rbits[lane + 32 * q];
#pragma unroll
            for (int p = 0; p < kBlrSketch; ++p) {
                const float sg = psign(hb, p);
                pr[p] = fmaf(sg, u.x, pr[p]);
                pi[p] = fmaf(sg, u.y, pi[p]);
            }
        }
#pragma unroll
        for (int p = 0; p < kBlrSketch; ++p) {
            pr[p] = warp_sumf(pr[p]);
            pi[p] = warp_sumf(pi[p]);
        }
        if (lane == 0)
#pragma unroll
            for (int p = 0; p < kBlrSketch; ++p) cw[p][l] = make_float2(pr[p], pi[p]);
    }
    __syncthreads();
    float2 acc0[kBlrSketch], acc1[kBlrSketch];
#pragma unroll
    for (int p = 0; p < kBlrSketch; ++p) acc0[p] = acc1[p] = make_float2(0.f, 0.f);
    float bn2 = 0.f;
    const int j = 2 * t;
    if (j < nc) {
        const float2 *col = A + (size_t)I0 * lda + J0 + j;
        const bool pair = j + 1 < nc;
#pragma unroll 8
        for (int i = 0; i < m; ++i) {
            const unsigned bits = rbits[i];
            float4 bv;
            if (pair) {
                bv = __ldcs(reinterpret_cast<const float4 *>(col + (size_t)i * lda));
            } else {
                const float2 v = __ldcs(col + (size_t)i * lda);
                bv = make_float4(v.x, v.y, 0.f, 0.f);
            }
            bn2 = fmaf(bv.x, bv.x, fmaf(bv.y, bv.y, bn2));
            bn2 = fmaf(bv.z, bv.z, fmaf(bv.w, bv.w, bn2));
#pragma unroll
            for (int p = 0; p < kBlrSketch; ++p) {
                const float sg = psign(bits, p);
                acc0[p].x = fmaf(sg, bv.x, acc0[p].x);
                acc0[p].y = fmaf(sg, bv.y, acc0[p].y);
                acc1[p].x = fmaf(sg, bv.z, acc1[p].x);
                acc1[p].y = fmaf(sg, bv.w, acc1[p].y);
            }
        }
    }
    for (int l = 0; l < k; ++l) {
        const float4 v = *reinterpret_cast<const float4 *>(V + (size_t)l * kBlrB + j);   // zero past the block
#pragma unroll
        for (int p = 0; p < kBlrSketch; ++p) {
            const float2 w0 = cmul2(cw[p][l], make_float2(v.x, v.y));
            const float2 w1 = cmul2(cw[p][l], make_float2(v.z, v.w));
            acc0[p].x -= w0.x;
            acc0[p].y -= w0.y;
            acc1[p].x -= w1.x;
            acc1[p].y -= w1.y;
        }
    }
    float est = 0.f;
#pragma unroll
    for (int p = 0; p < kBlrSketch; ++p) {
        est = fmaf(acc0[p].x, acc0[p].x, fmaf(acc0[p].y, acc0[p].y, est));
        est = fmaf(acc1[p].x, acc1[p].x, fmaf(acc1[p].y, acc1[p].y, est));
    }
    est = warp_sumf(est);
    bn2 = warp_sumf(bn2);
    if (lane == 0) {
        red[0][warp] = est;
        red[1][warp] = bn2;
    }
    // Frobenius norms of the terms, |U_l| |V_l| (warp w: terms w, w + 4, ...)
    for (int l = warp; l < k; l += kChkWarps) {
        float nu = 0.f, nv = 0.f;
#pragma unroll
        for (int q = 0; q < kBlrB / 32; ++q) {
            const float2 u = U[(size_t)l * kBlrB + lane + 32 * q], v = V[(size_t)l * kBlrB + lane + 32 * q];
            nu = fmaf(u.x, u.x, fmaf(u.y, u.y, nu));
            nv = fmaf(v.x, v.x, fmaf(v.y, v.y, nv));
        }
        nu = warp_sumf(nu);
        nv = warp_sumf(nv);
        if (lane == 0) tn[l] = sqrtf(nu) * sqrtf(nv);
    }
    __syncthreads();
    if (t == 0) {
        float e = 0.f, bb = 0.f;
        for (int w = 0; w < kChkWarps; ++w) {
            e += red[0][w];
            bb += red[1][w];
        }
        const float est = e / (float)kBlrSketch;
        keep = est <= kBlrTol * kBlrTol * bb;
        int kk = k;
        if (keep) {
            // drop trailing terms within half the tolerance left: by the
            // triangle inequality the error grows by at most their norms
            const float budget = 0.5f * (kBlrTol * sqrtf(bb) - sqrtf(est));
            float dropped = 0.f;
            while (kk > 0 && dropped + tn[kk - 1] <= budget) dropped += tn[--kk];
        }
        kept = kk;
        S.rank[b] = keep ? kk : -1;
    }
    __syncthreads();
    if (!keep) return;
    // the kept terms as fp16 factors, scale 2^(eu - 15) 2^(ev - 15) per term
    unsigned *U16 = S.U16 + (size_t)b * kBlrMaxRank * kBlrB;
    unsigned *V16 = S.V16 + (size_t)b * kBlrMaxRank * kBlrB;
    for (int l = warp; l < kept; l += kChkWarps) {
        const int eu = store_half(U + (size_t)l * kBlrB, U16 + (size_t)l * kBlrB, lane);
        const int ev = store_half(V + (size_t)l * kBlrB, V16 + (size_t)l * kBlrB, lane);
        if (lane == 0) S.scale[(size_t)b * kBlrMaxRank + l] = ldexpf(1.f, eu + ev - 30);
    }
}

}  // namespace

void blr_batch_finish(BlrBatch &t) {
    t.off[0] = 0;
    for (int b = 0; b < t.B; ++b) {
        const int nb = blr_blocks(t.sys[b].n);
        t.off[b + 1] = t.off[b] + nb * nb;
    }
}

cudaError_t launch_blr_compress(const BlrBatch &t, cudaStream_t st) {
    if (t.B <= 0 || t.off[t.B] == 0) return cudaSuccess;
    count_launches(2);
    const int grid = (t.off[t.B] + kBlrWarps - 1) / kBlrWarps;
    k_blr_aca<<<grid, 32 * kBlrWarps, 0, st>>>(t);
    k_blr_check<<<t.off[t.B], kChkThreads, 0, st>>>(t);
    return cudaGetLastError();
}

}  // namespace bem
