// bem_static.cu - bem_project_static: field projection that allocates no
// device memory.
//
// All of its scratch lives in the file-scope array below instead of in
// buffers owned by a solver or allocated per call: the element potentials,
// nodal velocities, their float copies and the nonzero-velocity flags the
// projection kernels need between their two launches, the error word, and
// the per-(element slice, point) partial sums of the float projection.  In
// host code the array's name is only a host-side stand-in, so the device
// address is looked up once per device with cudaGetSymbolAddress (with that
// device current) and that address is what the kernels receive.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/bem_gb300.h"
#include "bem_internal.h"

namespace {

constexpr int kStaticMaxElem = BEM_STATIC_MAX_ELEMENTS;
// per element: phi (16 B) + 4 nodal velocities (64 B) + their float copies
// (8 + 32 B) + flag (4 B); then the error word (256 B); then the partial
// sums of the float projection.  With fewer partial-sum slots than a call
// needs, the projection takes wider element slices, and below one slice per
// 32-point group it runs one warp per point (same quadrature, FP32 sums).
constexpr size_t kElemBytes = (size_t)kStaticMaxElem * (16 + 64 + 8 + 32 + 4);
constexpr size_t kPartBytes = (size_t)8 << 20;
constexpr size_t kScratchBytes = kElemBytes + 256 + kPartBytes;

static __device__ __align__(256) unsigned char g_project_scratch[kScratchBytes];

std::mutex g_mu;
void *g_addr[64];   // device address of g_project_scratch, per device

}  // namespace

namespace bem {
// accessors of the solver state, defined in bem_api.cu
bool solver_projection_inputs(bem_solver_t s, int max_elem, ProjSys *out, int *prec, int *device);
void set_error(const char *msg);
}  // namespace bem

extern "C" bem_status bem_project_static(bem_solver_t solver, int32_t n_pts, const double *pts_dev,
                                         double *pot_dev, double *grad_dev, void *stream) {
    bem::ProjBatch t;
    int prec = 0, mesh_dev = -1;
    if (!bem::solver_projection_inputs(solver, kStaticMaxElem, &t.sys[0], &prec, &mesh_dev)) return BEM_ERR_INVALID;
    if (n_pts < 0 || (n_pts > 0 && (!pts_dev || !pot_dev))) {
        bem::set_error("bem_project_static: bad point or output pointers");
        return BEM_ERR_INVALID;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        bem::set_error("bem_project_static: no current CUDA device");
        return BEM_ERR_CUDA;
    }
    // the scratch address, the solver's tables and the stream must all belong
    // to one device: the one the solver's mesh lives on
    if (dev != mesh_dev) {
        bem::set_error("bem_project_static: the current CUDA device is not the solver's device");
        return BEM_ERR_INVALID;
    }
    cudaStream_t st = (cudaStream_t)stream;
    int st_dev = -1;
    if (cudaStreamGetDevice(st, &st_dev) != cudaSuccess || st_dev != mesh_dev) {
        cudaGetLastError();
        bem::set_error("bem_project_static: the stream does not belong to the solver's device");
        return BEM_ERR_INVALID;
    }
    void *base = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (!g_addr[dev]) {
            void *p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_project_scratch);
            if (e != cudaSuccess) {
                bem::set_error(cudaGetErrorString(e));
                return BEM_ERR_CUDA;
            }
            g_addr[dev] = p;
        }
        base = g_addr[dev];
    }
    unsigned char *b = (unsigned char *)base;
    int *status = (int *)(b + kElemBytes);
    // the fields kernel indexes vel as [4][n] with row stride n, so the
    // scratch layout holds for any n up to the maximum
    bem::ProjSys &S = t.sys[0];
    S.phi = (double *)b;
    S.vel = (double *)(b + (size_t)kStaticMaxElem * 16);
    S.phi32 = (float *)(b + (size_t)kStaticMaxElem * 80);
    S.vel32 = (float *)(b + (size_t)kStaticMaxElem * 88);
    S.ivi = (int *)(b + (size_t)kStaticMaxElem * 120);
    S.status = status;
    S.part = (float4 *)(b + kElemBytes + 256);
    S.part_cap = (long long)(kPartBytes / sizeof(float4));
    S.npts = n_pts;
    S.pts = pts_dev;
    S.pot = pot_dev;
    S.grad = grad_dev;
    t.B = 1;
    bem::proj_batch_finish(t);
    cudaError_t e = cudaMemsetAsync(status, 0, sizeof(int), st);
    if (e == cudaSuccess) e = bem::launch_fields(t, st);
    if (e == cudaSuccess && n_pts > 0) e = bem::launch_project(t, prec, st);
    int st_h = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&st_h, status, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        bem::set_error(cudaGetErrorString(e));
        return BEM_ERR_CUDA;
    }
    if (st_h != 0) {
        bem::set_error("evaluation point too close to the boundary: subdivision limit");
        return BEM_ERR_SUBDIVISION;
    }
    return BEM_OK;
}
