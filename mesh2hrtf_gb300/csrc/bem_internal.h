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
    const float *chi, *clo, *t32, *q32, *isqa32;
};

// One frequency's data on the device.
struct DevFreq {
    double k, wr, tao, beta_im;
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

// Process-wide count of kernel launches issued by the launch_* functions.
void count_launches(int k);
long long launches();

// Copies the quadrature tables into constant memory of the current device.
cudaError_t init_device_tables();

// A = assembled TBEM matrix, row-major n x n with leading dimension lda,
// complex128 (prec 0) or complex64 (prec 1).  status: device int receiving
// subdivision errors.
cudaError_t launch_assemble(const DevMeshView &m, const DevFreq &f, int prec, void *A, size_t lda, int *status,
                            unsigned long long *n_near, cudaStream_t st);
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
                          const double *r_in, double *y, void *xf, cudaStream_t st);
// h[l] = <V[l], w> (conjugated in V) for l < nv; V has leading dimension ldv.
cudaError_t launch_multi_dot(const double *V, int ldv, int nv, const double *w, int n, double *h,
                             cudaStream_t st);
// w -= sum_l h[l] V[l];  optionally hacc[l] += h[l].
cudaError_t launch_multi_axpy(const double *V, int ldv, int nv, const double *h, double *hacc, double *w,
                              int n, cudaStream_t st);
// out[0] = ||w||^2
cudaError_t launch_norm2(const double *w, int n, double *out, cudaStream_t st);
// v = w * (1 / sqrt(nrm2[0]))
cudaError_t launch_scale_inv(const double *w, const double *nrm2, double *v, int n, cudaStream_t st);
// x += sum_l y[l] V[l]  (y complex on the device)
cudaError_t launch_update_x(const double *V, int ldv, int nv, const double *y, double *x, int n,
                            cudaStream_t st);

}  // namespace bem
