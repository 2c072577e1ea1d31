// bem_static.cu - bem_project_static: field projection that allocates no
// device memory.
//
// Its scratch (element potentials, nodal velocities, the nonzero-velocity
// flags and the error word the projection kernels need between their two
// launches) lives in the file-scope array below instead of in buffers owned
// by a solver or allocated per call.  In host code the array's name is only a
// host-side stand-in, so the device address is looked up once per device with
// cudaGetSymbolAddress (with that device current) and that address is what
// the kernels receive.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/bem_gb300.h"
#include "bem_internal.h"

namespace {

constexpr int kStaticMaxElem = BEM_STATIC_MAX_ELEMENTS;
// per element: phi (16 B) + 4 nodal velocities (64 B) + their float copies
// (8 + 32 B) + flag (4 B), then the error word
constexpr size_t kScratchBytes = (size_t)kStaticMaxElem * (16 + 64 + 8 + 32 + 4) + 256;

static __device__ __align__(256) unsigned char g_project_scratch[kScratchBytes];

std::mutex g_mu;
void *g_addr[64];   // device address of g_project_scratch, per device

}  // namespace

namespace bem {
// accessors of the solver state, defined in bem_api.cu
bool solver_projection_inputs(bem_solver_t s, int max_elem, ProjSys *out, int *prec);
void set_error(const char *msg);
}  // namespace bem

extern "C" bem_status bem_project_static(bem_solver_t solver, int32_t n_pts, const double *pts_dev,
                                         double *pot_dev, double *grad_dev, void *stream) {
    bem::ProjBatch t;
    int prec = 0;
    if (!bem::solver_projection_inputs(solver, kStaticMaxElem, &t.sys[0], &prec)) return BEM_ERR_INVALID;
    if (n_pts < 0 || (n_pts > 0 && (!pts_dev || !pot_dev))) {
        bem::set_error("bem_project_static: bad point or output pointers");
        return BEM_ERR_INVALID;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        bem::set_error("bem_project_static: no current CUDA device");
        return BEM_ERR_CUDA;
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
    cudaStream_t st = (cudaStream_t)stream;
    unsigned char *b = (unsigned char *)base;
    int *status = (int *)(b + (size_t)kStaticMaxElem * 124);
    // the fields kernel indexes vel as [4][n] with row stride n, so the
    // scratch layout holds for any n up to the maximum
    bem::ProjSys &S = t.sys[0];
    S.phi = (double *)b;
    S.vel = (double *)(b + (size_t)kStaticMaxElem * 16);
    S.phi32 = (float *)(b + (size_t)kStaticMaxElem * 80);
    S.vel32 = (float *)(b + (size_t)kStaticMaxElem * 88);
    S.ivi = (int *)(b + (size_t)kStaticMaxElem * 120);
    S.status = status;
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
