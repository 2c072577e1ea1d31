// bem_solver.h - handles of the C ABI (mesh, solver) and the group
// operations shared by the single-solver, batched and served entry points
// (bem_api.cu, bem_server.cu).
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <vector>

#include "../../include/bem_gb300.h"
#include "bem_engine.h"
#include "bem_internal.h"

namespace bem {
// Sets the calling thread's error message; returns st.
bem_status fail(bem_status st, const char *fmt, ...);
inline size_t round_up(size_t v, size_t a) { return (v + a - 1) / a * a; }
}  // namespace bem

#define BEM_CU(call)                                                                             \
    do {                                                                                         \
        cudaError_t e_ = (call);                                                                 \
        if (e_ != cudaSuccess)                                                                   \
            return bem::fail(BEM_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
    } while (0)

// Device-resident mesh (bem_mesh_create).
struct bem_mesh_s {
    int device = 0;
    int n = 0;
    std::vector<int> nvert;         // internal order
    std::vector<int> ext_of_int;    // internal unknown -> caller's element index
    std::vector<int> int_of_ext;
    // device buffers
    int *d_nvert = nullptr;
    double *d_v64 = nullptr, *d_c64 = nullptr, *d_n64 = nullptr, *d_area = nullptr, *d_sqa = nullptr;
    float *d_chi = nullptr, *d_clo = nullptr, *d_t32 = nullptr, *d_q32 = nullptr, *d_isqa = nullptr;
    float *d_n32 = nullptr;
    float4 *d_row4 = nullptr;
    int2 *d_near = nullptr;         // pairs integrated with subdivision + self pairs
    long long n_near = 0;
    bem::DevSym sym{};              // symmetry-plane images (sym.nref = 1: none)
    void *d_img = nullptr;          // one allocation holding the image tables
    bem::DevMeshView view() const {
        bem::DevMeshView v;
        v.n = n; v.nvert = d_nvert; v.v64 = d_v64; v.c64 = d_c64; v.n64 = d_n64; v.area64 = d_area;
        v.sqa64 = d_sqa; v.chi = d_chi; v.clo = d_clo; v.t32 = d_t32; v.q32 = d_q32; v.isqa32 = d_isqa;
        v.n32 = d_n32;
        v.row4 = d_row4;
        v.sym = sym;
        return v;
    }
    ~bem_mesh_s() {
        for (void *p : {(void *)d_nvert, (void *)d_v64, (void *)d_c64, (void *)d_n64, (void *)d_area, (void *)d_sqa,
                        (void *)d_chi, (void *)d_clo, (void *)d_t32, (void *)d_q32, (void *)d_isqa, (void *)d_near,
                        (void *)d_n32, (void *)d_row4, d_img})
            bem::dev_free(p);
    }
};

namespace bem {

// Sources kept in the solver's block; more are allocated separately.
constexpr int kInlineSources = 64;

// Every per-solver device buffer, carved from one allocation.
struct SolverBufs {
    void *A = nullptr;
    void *A16 = nullptr;       // mixed precision, one right-hand side: fp16 copy of A
    float *rs = nullptr;       // its row scales
    int blr_nb = 0;            // mixed precision, one right-hand side: block low-rank
    int *blr_rank = nullptr;   // copy of A (kBlrB blocks, blr_nb per row; BlrSys)
    float2 *blr_U = nullptr, *blr_V = nullptr;   // for the Krylov products
    unsigned *blr_U16 = nullptr, *blr_V16 = nullptr;
    float *blr_scale = nullptr;
    double2 *b = nullptr, *x = nullptr, *r = nullptr, *w = nullptr, *z = nullptr, *V = nullptr;
    double2 *mvp = nullptr, *dpa = nullptr, *dpb = nullptr;
    float2 *xh = nullptr;
    float4 *xf = nullptr;
    double *nrmp = nullptr;
    double2 *H = nullptr, *cs = nullptr, *sn = nullptr, *g = nullptr, *y = nullptr, *hsum = nullptr;
    void *Minv = nullptr, *Mwork = nullptr;
    void *pcy = nullptr, *pcz = nullptr;   // window correction vectors
    int *status = nullptr;
    unsigned *ctr = nullptr;   // 4 words: work queues of the persistent assembly kernels
    double *phi = nullptr, *vel = nullptr;
    float *phi32 = nullptr, *vel32 = nullptr;
    int *ivi = nullptr;
    int *bct = nullptr, *cols = nullptr;
    double *bcv = nullptr, *adm = nullptr, *src = nullptr;
};

// Byte layout of a solver's block for n_rhs right-hand sides; base ==
// nullptr only sizes it (bem_footprint_bytes is this size for one).
// krylov_copy: the copy of A that the Krylov products of complex64 solvers
// with one right-hand side read: 0 fp16 (row-scaled), 1 none (they read A),
// 2 block low-rank over the fp16 copy.
size_t solver_layout(int n, int prec, int m, bool pc, unsigned char *base, SolverBufs *o, int n_rhs = 1,
                     SolverBufs *extra = nullptr, int krylov_copy = 0);

}  // namespace bem

struct bem_solver_s {
    bem_mesh_t mesh = nullptr;
    int n = 0;
    int prec = 0;
    int restart = 60;
    int max_iter = 1000;
    double tol = 1e-9;
    size_t lda = 0;
    bool precond = true, have_precond = false;
    bool pc_window = true;   // block-Jacobi with the window correction step
    bool pc_scaling = false; // NumCalc's diagonal scaling instead of block-Jacobi
    cudaStream_t st = nullptr;
    cudaEvent_t ev[8] = {};
    unsigned char *block = nullptr;
    size_t block_bytes = 0;
    bem::SolverBufs d;                     // right-hand side 0 and the shared buffers
    int n_rhs = 1;
    std::vector<bem::SolverBufs> xr;       // right-hand sides 1 .. n_rhs-1
    std::vector<bem::DevFreq> xfreq;       // their frequency data (sources, boundary values)
    double *src_extra = nullptr;
    bem::DevFreq freq{};
    bool have_freq = false;
    bool factored = false;    // A holds LU factors (bem_solve_direct) until the next assembly
    int mv_strip = 0;         // rows per item of the complex64 product (0: default; tuner's choice)
    bool solved = false;
    double *pts = nullptr, *pot = nullptr, *grad = nullptr;
    int pts_cap = 0;
    bool own_block = true;    // false: block and point buffers belong to a server's arena
    std::unique_ptr<bem::Engine> eng;
    bem_solve_info info{};
    ~bem_solver_s() {
        if (st) cudaStreamSynchronize(st);
        eng.reset();
        if (own_block) {
            bem::dev_free(block);
            bem::dev_free(pts); bem::dev_free(pot); bem::dev_free(grad);
        }
        bem::dev_free(src_extra);
        for (auto &e : ev)
            if (e) cudaEventDestroy(e);
        if (st) cudaStreamDestroy(st);
    }
    const bem::SolverBufs &buf(int r) const { return r == 0 ? d : xr[r - 1]; }
    const bem::DevFreq &fq(int r) const { return r == 0 ? freq : xfreq[r - 1]; }
    bem::KSys ksys(int r = 0) const {
        const bem::SolverBufs &d = buf(r);
        bem::KSys k{};
        k.A = d.A;
        k.A16 = d.A16;
        k.rs = d.rs;
        k.cgs1 = 0;   // the float basis of complex64 systems needs the second pass
        k.lda = (long long)lda;
        k.n = n;
        k.pc = have_precond ? 1 : 0;
        k.pcw = have_precond && pc_window ? 1 : 0;
        k.pcy = d.pcy;
        k.pcz = d.pcz;
        k.nchunk = bem::mv_chunks(n);
        k.nvb = bem::vec_blocks(n);
        k.Minv = d.Minv;
        k.x = d.x; k.b = d.b; k.r = d.r; k.w = d.w; k.z = d.z; k.V = d.V;
        k.xh = d.xh; k.xf = d.xf;
        k.ldv = n;
        k.mvp = d.mvp; k.dpa = d.dpa; k.dpb = d.dpb; k.nrmp = d.nrmp;
        k.H = d.H; k.cs = d.cs; k.sn = d.sn; k.g = d.g; k.y = d.y; k.hsum = d.hsum;
        k.strip = mv_strip;
        k.blr_nb = d.blr_nb;
        k.blr_rank = d.blr_rank;
        k.blr_U16 = d.blr_U16;
        k.blr_V16 = d.blr_V16;
        k.blr_scale = d.blr_scale;
        return k;
    }
    bem::KState kinit() const {
        bem::KState q{};
        q.phase = bem::kPhaseUpdate;
        q.m = restart;
        q.max_iter = max_iter;
        q.tol = tol;
        // inner cycles stop at this fraction of the cycle's starting residual:
        // with the fp16 Krylov copy (perturbation ~5e-4 relative) a cycle
        // gains about three digits on the complex64 system; 3e-4 rather than
        // 1e-3 saves a refinement cycle now and then for a few more steps
        // (the right-hand sides of a solver with several share TF32 tensor-core
        // products of about the same accuracy)
        const bool tf32 = n_rhs > 1 && bem::group_product_umma();
        q.floor_rel = prec == BEM_PREC_MIXED ? ((d.A16 || d.blr_nb > 0 || tf32) ? 3e-4 : 1e-5) : 0.0;
        return q;
    }
    bem::AsmSys asys(int r = 0) const {
        const bem::SolverBufs &d = buf(r);
        bem::AsmSys a{};
        a.m = mesh->view();
        a.f = fq(r);
        a.A = d.A;
        a.lda = lda;
        a.near = mesh->d_near;
        a.n_near = mesh->n_near;
        a.b = (double *)d.b;
        a.status = d.status;
        return a;
    }
    bem::PcSys psys() const {
        bem::PcSys p{};
        p.A = d.A;
        p.lda = lda;
        p.n = n;
        p.Minv = d.Minv;
        p.work = d.Mwork;
        p.status = d.status;
        return p;
    }
    bem::ProjSys prsys(int npts, const double *pts_dev, double *pot_dev, double *grad_dev, int r = 0) const {
        const bem::SolverBufs &d = buf(r);
        bem::ProjSys q{};
        q.m = mesh->view();
        q.f = fq(r);
        q.x = (const double *)d.x;
        q.phi = d.phi;
        q.vel = d.vel;
        q.phi32 = d.phi32;
        q.vel32 = d.vel32;
        q.ivi = d.ivi;
        q.npts = npts;
        q.pts = pts_dev;
        q.pot = pot_dev;
        q.grad = grad_dev;
        q.status = d.status;
        q.part = reinterpret_cast<float4 *>(d.V);
        q.part_cap = (long long)((size_t)(restart + 1) * (size_t)n * (prec == BEM_PREC_FP64 ? 16 : 8) / 16);
        return q;
    }
};

namespace bem {

// Frequency data into the solver's block (internal element order); rhs > 0
// takes only the boundary values and sources of right-hand side rhs (the
// matrix data comes from right-hand side 0).
bem_status upload_freq(bem_solver_t s, const bem_frequency_desc *f, cudaStream_t st, int rhs = 0);
// Map a finished GMRES state to a status (and message).
bem_status map_result(const KState &q);
// Assembly + right-hand side of every solver in ss (frequencies uploaded).
bem_status assemble_group(bem_solver_t *ss, int cnt, cudaStream_t st, unsigned *ctr, cudaEvent_t e0,
                          cudaEvent_t e1, bem_status *rcs);
// Block-Jacobi inverses of every preconditioned solver in ss and x = 0.
bem_status precond_group(bem_solver_t *ss, int cnt, cudaStream_t st);
// fp16 Krylov copies of the complex64 matrices of ss that keep one.
cudaError_t split_group(bem_solver_t *ss, int cnt, cudaStream_t st);
// Restarted GMRES of every solver in ss until all have finished.
bem_status solve_group(bem_solver_t *ss, int cnt, Engine *eng, cudaStream_t st, cudaEvent_t e0, cudaEvent_t e1,
                       bem_status *rcs);
// Fields and projection of every solver in ss (points from the host).
bem_status project_group(bem_solver_t *ss, int cnt, const int32_t *npts, const double *const *pts,
                         double *const *pot_out, double *const *grad_out, cudaStream_t st, cudaEvent_t e0,
                         cudaEvent_t e1, bem_status *rcs);
// Unknowns to host memory in the caller's element order.
bem_status solution_to_host(bem_solver_t s, cudaStream_t st, double *x_host, int rhs = 0);

}  // namespace bem
