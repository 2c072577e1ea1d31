// bem_internal.h - host-side interface between the C ABI (bem_api.cu) and the
// kernel translation units (bem_kernels.cu, bem_krylov.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace bem {

// Device element tables; layout documented in bem_common.cuh (DevMesh).
struct DevMeshView {
    int n;
    const int *nvert;
    const double *v64, *c64, *n64, *area64, *sqa64;
    const float *chi, *clo, *t32, *q32, *isqa32, *n32;
};

// One frequency's data on the device.
struct DevFreq {
    double k, wr, tao, beta_im;
    float kf, wrf, taof, beta_imf;   // the same in float
    const int *bc_type;        // [n] or nullptr (all velocity)
    const double *bc_val;      // [4][n] complex (row a = node a), or nullptr
    const double *adm;         // [n] complex, or nullptr
    const int *bc_cols;        // columns with nonzero prescribed values
    int n_bc_cols;
    int n_point, n_plane;
    const double *ps_xyz;      // [n_point][3]
    const double *ps_amp;      // [n_point] complex
    const double *pw_dir;      // [n_plane][3]
    const double *pw_amp;      // [n_plane] complex
};

// Unknowns per diagonal block of the block-Jacobi preconditioner.
constexpr int kBlock = 128;

// Process-wide count of kernel launches issued by the launch_* functions.
void count_launches(int k);
long long launches();

// Copies the quadrature tables into constant memory of the current device.
cudaError_t init_device_tables();

// Pairs integrated with subdivision plus self pairs, (row, column);
// list == nullptr only counts.
cudaError_t launch_near_list(const DevMeshView &m, int2 *list, unsigned long long *count, cudaStream_t st);
// A = assembled TBEM matrix, row-major n x n with leading dimension lda,
// complex128 (prec 0) or complex64 (prec 1): regular pairs, then the near
// list.  status: device int receiving subdivision errors.
cudaError_t launch_assemble(const DevMeshView &m, const DevFreq &f, int prec, void *A, size_t lda,
                            const int2 *near_list, long long n_near, int *status, cudaStream_t st);
// b = free terms + incident waves + columns with prescribed values (FP64).
cudaError_t launch_rhs(const DevMeshView &m, const DevFreq &f, double *b, int *status, cudaStream_t st);
// Element potentials and nodal normal velocities from the unknowns x.
cudaError_t launch_fields(const DevMeshView &m, const DevFreq &f, const double *x, double *phi,
                          double *vel, int *ivi, cudaStream_t st);
// Potential and gradient at npts points (pts: [npts][3] FP64 on the device).
cudaError_t launch_project(const DevMeshView &m, const DevFreq &f, int prec, const double *phi,
                           const double *vel, const int *ivi, int npts, const double *pts,
                           double *pot, double *grad, int *status, cudaStream_t st);

// ---- Krylov building blocks (bem_krylov.cu); vectors are complex128 ----
// Device-side control word of one GMRES cycle.  Kernels given `done` return
// at once when it is set, so the host can queue several Arnoldi steps ahead
// and check convergence once per batch.
struct GmresCtrl {
    int done;     // residual estimate reached thr (or breakdown)
    int kdone;    // Arnoldi steps completed in this cycle
    double res;   // |g[k+1]| after the last step
    double thr;   // absolute residual target of the cycle
};

// y = A x for a row-major n x n matrix with leading dimension lda
// (r_in != nullptr: y = r_in - A x).
// prec 0: complex128 A, FP64 arithmetic.
// prec 1, exact = false: complex64 A, x rounded to complex64, FP32 products
//   and per-lane sums, FP64 reduction across lanes (Krylov inner products).
// prec 1, exact = true: complex64 A times x = x_hi + x_lo with error-free
//   products (FMA two-product) and two-sum accumulation, i.e. twice-FP32
//   accuracy (the refinement residual).
// xf: scratch of 2 * n float2 for the split of x.
cudaError_t launch_matvec(int prec, bool exact, const void *A, int n, size_t lda, const double *x,
                          const double *r_in, double *y, void *xf, cudaStream_t st, const int *done = nullptr);
// Blocks of partial sums used by launch_multi_dot.
int dot_blocks(int n);
// h[l] = <V[l], w> (conjugated in V) for l < nv, V with leading dimension
// ldv (complex entries); hsum[l] += h[l] if hsum != nullptr.  partial: nv *
// dot_blocks(n) complex scratch.
cudaError_t launch_multi_dot(const double *V, size_t ldv, int nv, const double *w, int n, double *partial,
                             double *h, double *hsum, cudaStream_t st, const int *done = nullptr);
// w -= sum_l h[l] V[l]
cudaError_t launch_multi_axpy(const double *V, size_t ldv, int nv, const double *h, double *w, int n,
                              cudaStream_t st, const int *done = nullptr);
// out[0] = ||w||^2
cudaError_t launch_norm2(const double *w, int n, double *out, cudaStream_t st);
// v = w * (1 / sqrt(nrm2[0]))
cudaError_t launch_scale_inv(const double *w, const double *nrm2, double *v, int n, cudaStream_t st,
                             const int *done = nullptr);
// Givens step k of the cycle on the device (see GmresCtrl).
cudaError_t launch_givens(int k, int m, double *hsum, const double *wnorm2, double *H, double *cs, double *sn,
                          double *g, GmresCtrl *ctrl, cudaStream_t st);
// x += sum_l y[l] V[l]  (y complex on the device)
cudaError_t launch_update_x(const double *V, int ldv, int nv, const double *y, double *x, int n,
                            cudaStream_t st);

// ---- block-Jacobi preconditioner (bem_precond.cu) ----
size_t precond_bytes(int n, int prec);
// Inverts the kBlock x kBlock diagonal blocks of A into Minv (transposed
// blocks); FP64 uses `work` (same size as Minv) as inversion workspace.
cudaError_t launch_block_inverse(int prec, const void *A, size_t lda, int n, void *Minv, void *work, int *status,
                                 cudaStream_t st);
// z = M^{-1} v
cudaError_t launch_block_apply(int prec, const void *Minv, int n, const double *v, double *z, cudaStream_t st,
                               const int *done = nullptr);
// x += z
cudaError_t launch_axpy(const double *z, double *x, int n, cudaStream_t st);

}  // namespace bem
