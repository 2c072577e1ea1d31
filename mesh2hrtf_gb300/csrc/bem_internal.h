// bem_internal.h - host-side interface between the C ABI (bem_api.cu, the
// engine) and the kernel translation units (bem_kernels.cu, bem_gmres.cu,
// bem_precond.cu).
//
// Every launch is batched: it works on a table of systems ((mesh, frequency)
// instances), and a single solve is a batch of one.  Assembly, right-hand
// side, preconditioner set-up and projection take their table by value (kernel
// parameter space, __grid_constant__); the Krylov kernels read theirs from
// device memory so that one captured CUDA graph serves any composition of the
// batch.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace bem {

// Images of the elements in up to three symmetry planes (NumCalc's SYMMETRY
// block).  Image kref = 1 .. nref-1 is image kref-1 reflected once, across
// the plane normal to axis rdir[kref] (the reference's Gray-code order,
// NC_3dFunctions.cpp:181-242,357-452); its vertices are stored in the
// reference's node order after the reflections (nodes 0/1 and 2/3 swapped
// for odd kref).
struct DevSym {
    int nref;                 // images per element: 1, 2, 4 or 8
    unsigned rneg;            // bit kref: the reflection factor of image kref is -1
    unsigned axes;            // bit k: a plane is normal to axis k
    unsigned char rdir[8];    // axis reflected in step kref (1 .. nref-1)
    double coord[3];          // plane positions on the axes
    // tables of images 1 .. nref-1, each laid out like the mesh's own
    // (stride n); image kref starts at (kref - 1) * rows * n
    const double *v64, *c64;
    const float *chi, *clo, *t32, *q32;
};

// Device element tables; layout documented in bem_common.cuh (DevMesh).
struct DevMeshView {
    int n;
    const int *nvert;
    const double *v64, *c64, *n64, *area64, *sqa64;
    const float *chi, *clo, *t32, *q32, *isqa32, *n32;
    const float4 *row4;     // [n][3]: (chi, 0), (clo, 0), (n32, 0) of each element
    DevSym sym;
};

// Near-list entries are (row, column | image mask << 24): bit kref of the
// mask marks image kref of the column element as integrated with
// subdivision (or, for kref = 0 on the diagonal, the singular integral).
constexpr int kNearColBits = 24;
constexpr int kMaxElements = (1 << kNearColBits) - 1;

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
// Rows of a window of the preconditioner's correction step (8 blocks): the
// preconditioner is M = X (2 I - A_w X), X the block-Jacobi inverse and A_w
// the diagonal windows of A (one Neumann step towards the inverse of A_w).
constexpr int kPcWin = 1024;
// Rows per block of the vector kernels (two preconditioner blocks).
constexpr int kVecBlock = 256;
// Matrix-vector product tile: kMvRows rows x kMvChunk columns.
constexpr int kMvRows = 32;
constexpr int kMvChunk = 1024;
// Largest GMRES restart length (basis of kMaxRestart + 1 vectors).
constexpr int kMaxRestart = 63;
// Systems per launch table.
constexpr int kMaxAsm = 64;    // assembly / projection / preconditioner set-up
constexpr int kMaxSys = 128;   // Krylov engine slots
constexpr int kMaxRhs = 16;    // right-hand sides of one solver

__host__ __device__ inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }
__host__ __device__ inline int mv_chunks(int n) { return ceil_div(n, kMvChunk); }
inline int vec_blocks(int n) { return ceil_div(n, kVecBlock); }
inline int pc_blocks(int n) { return ceil_div(n, kBlock); }

// Process-wide count of kernel launches issued by the launch_* functions.
void count_launches(long long k);
// Sets the calling thread's error message (bem_last_error).
void set_error(const char *msg);
long long launches();

// Device-memory cache for meshes, solvers and point buffers.  Released blocks
// stay allocated per device and go to the next request of about the same size
// (at most 1/8 larger): cudaFree synchronizes the device and takes
// milliseconds for GB-sized blocks, so creating and destroying solvers per
// request would otherwise cost as much as a small solve.  dev_free waits for
// the device to be idle before keeping a block, as cudaFree does.  A failed
// cudaMalloc releases the cached blocks and retries.  BEM_GB300_CACHE=0 turns
// the cache off.
cudaError_t dev_malloc(void **p, size_t bytes);
void dev_free(void *p);
size_t dev_cached_bytes(int device);
void dev_release_cached(int device);   // device < 0: every device

// Copies the quadrature tables into constant memory of the current device.
cudaError_t init_device_tables();

// ---------------------------------------------------------------- assembly
struct AsmSys {
    DevMeshView m;
    DevFreq f;
    void *A;                // row-major n x n, leading dimension lda
    size_t lda;
    const int2 *near;       // near list of the mesh: (row, column)
    long long n_near;
    double *b;              // right-hand side (complex)
    int *status;            // subdivision errors (atomicMax)
};
struct AsmBatch {
    int B;
    int img;                     // some system's mesh has symmetry images
    int far_off[kMaxAsm + 1];    // tiles of 32 x 32 entries
    int near_off[kMaxAsm + 1];   // near pairs
    int rhs_off[kMaxAsm + 1];    // blocks of 8 rows
    AsmSys sys[kMaxAsm];
};
// Fills the offset tables from sys[0..B).
void asm_batch_finish(AsmBatch &t);

// Pairs integrated with subdivision plus self pairs (row, column | image
// mask << kNearColBits) into list[0, cap); *count (zero before) receives the
// number of pairs, also when it exceeds cap.  scratch: device memory of
// near_list_scratch_bytes(n, nref) for the column blocks' bounding spheres.
size_t near_list_scratch_bytes(int n, int nref);
cudaError_t launch_near_list(const DevMeshView &m, void *scratch, int2 *list, unsigned long long cap,
                             unsigned long long *count, cudaStream_t st);
// Writable image tables of a mesh (DevSym's layout).
struct ImageTables {
    double *v64, *c64;
    float *chi, *clo, *t32, *q32;
};
// Fills the image tables of m (m.sym.nref > 1) from the mesh's own tables.
cudaError_t launch_image_tables(const DevMeshView &m, const ImageTables &out, cudaStream_t st);
// Device bytes of the image tables of n elements with nref images.
inline size_t image_table_bytes(int n, int nref) {
    return (size_t)(nref - 1) * (size_t)n * (15 * sizeof(double) + 28 * sizeof(float));
}
// A = assembled TBEM matrices of the batch, complex128 (prec 0) or complex64
// (prec 1): regular pairs (persistent k_far), then the near lists (persistent
// k_near).  ctr: 4 device words, zero before the first use; the kernels leave
// them zero.
// Launch shapes of the assembly (persistent grids: resident blocks per SM of
// k_far, at most kFarPerSmMax, and of k_near, at most 2); the results do not
// depend on them.
struct AsmShape {
    int far_per_sm = 3;
    int near_per_sm = 2;
};
constexpr int kFarPerSmMax = 3;
cudaError_t launch_assemble(const AsmBatch &t, int prec, unsigned *ctr, cudaStream_t st,
                            AsmShape shape = AsmShape());

// b = free terms + incident waves + columns with prescribed values (FP64).
cudaError_t launch_rhs(const AsmBatch &t, cudaStream_t st);

// ---------------------------------------------------------------- projection
struct ProjSys {
    DevMeshView m;
    DevFreq f;
    const double *x;        // solution (complex)
    double *phi, *vel;      // scratch: element potentials [n], nodal velocities [4][n]
    float *phi32, *vel32;   // the same in float (read by the float projection)
    int *ivi;               // [n] nonzero-velocity flags
    int npts;
    const double *pts;      // [npts][3]
    double *pot, *grad;     // [npts], [npts][3] complex; grad may be nullptr
    int *status;
    float4 *part;           // float projection: partial sums [slice][point][2]
                            // (the Krylov basis, idle once the system is solved)
    long long part_cap;     // its capacity in float4
    int nslice;             // element slices (proj_batch_finish; 0: one warp per point)
};
struct ProjBatch {
    int B;
    int fld_off[kMaxAsm + 1];    // blocks of 256 elements
    int pt_off[kMaxAsm + 1];     // blocks of 8 points
    int lp_off[kMaxAsm + 1];     // blocks of 8 (32-point group, element slice) warps
    int ps_off[kMaxAsm + 1];     // blocks of 256 points (slice sums)
    ProjSys sys[kMaxAsm];
};
void proj_batch_finish(ProjBatch &t);
// Element potentials and nodal normal velocities from the unknowns, then
// potential and gradient at the points.
cudaError_t launch_fields(const ProjBatch &t, cudaStream_t st);
cudaError_t launch_project(const ProjBatch &t, int prec, cudaStream_t st);
// The right-hand sides (systems 0 .. B-1, 2 <= B <= 8) of one complex64
// solver: kernel evaluations shared between them (falls back to
// launch_project when they do not share mesh, points and slicing).
cudaError_t launch_project_multi(const ProjBatch &t, cudaStream_t st);

// ---------------------------------------------------------------- preconditioner
struct PcSys {
    const void *A;
    size_t lda;
    int n;
    void *Minv;             // pc_blocks(n) blocks of kBlock x kBlock, transposed
    void *work;             // FP64 only: inversion workspace of the same size
    int *status;            // 1: a singular block
};
struct PcBatch {
    int B;
    int off[kMaxAsm + 1];
    PcSys sys[kMaxAsm];
};
void pc_batch_finish(PcBatch &t);
size_t precond_bytes(int n, int prec);
cudaError_t launch_block_inverse(const PcBatch &t, int prec, cudaStream_t st);
// NumCalc's scaling preconditioner in the block-Jacobi storage: Minv set to
// the diagonal d_i = sqrt(n / sum_j |a_ij|^2) (a zero row sets *status)
cudaError_t launch_pc_scaling(const PcSys &s, int prec, cudaStream_t st);

// ---------------------------------------------------------------- fp16 Krylov copy
// A complex64 system may also hold A in fp16 pairs, every row segment of
// kMvChunk columns scaled by a power of two that puts its largest component
// in [2^14, 2^15).  The Krylov
// products read that copy (4 bytes per entry instead of 8); the refinement
// residuals read the complex64 matrix, so the solution still meets the
// residual target with the complex64 system.
struct SplitSys {
    const void *A;          // complex64, leading dimension lda
    size_t lda;
    int n;
    void *A16;              // fp16 pairs, the same leading dimension
    float *rs;              // [n][mv_chunks(n)] segment scales:
                            // A[i][j] ~ rs[i * mv_chunks(n) + j / kMvChunk] * A16[i][j]
    const int *blr_rank;    // block low-rank copy's ranks (BlrSys::rank) or nullptr:
    int blr_nb;             // then only the segments read are converted: the
                            // diagonal chunk and chunks with a dense block
};
struct SplitBatch {
    int B;
    int off[kMaxAsm + 1];   // blocks (kSplitWarps segments each)
    SplitSys sys[kMaxAsm];
};
void split_batch_finish(SplitBatch &t);
cudaError_t launch_split16(const SplitBatch &t, cudaStream_t st);

// Block low-rank Krylov copy of a complex64 matrix (bem_blr.cu), with its
// fp16 copy for the blocks that stay dense: blocks of kBlrB x kBlrB unknowns.  Every off-diagonal block
// is approximated by adaptive cross approximation (stopping at kBlrStop);
// when a randomized estimate of the approximation's error (kBlrSketch
// Rademacher probes of the whole block) is within kBlrTol of the block's
// Frobenius norm, and at most kBlrMaxRank terms were needed, the block is
// kept as sum_l s_l U_l V_l^T with fp16 factors U_l, V_l and a power-of-two
// scale s_l; every other block (the diagonal ones included) is read from the
// fp16 copy.  The Krylov products read this copy; the refinement residuals
// keep reading A, so its accuracy bounds only how much an inner cycle gains.
constexpr int kBlrB = 256;
constexpr int kBlrMaxRank = 48;
constexpr float kBlrTol = 2e-4f;
constexpr float kBlrStop = 4e-5f;
constexpr int kBlrSketch = 8;
__host__ __device__ inline int blr_blocks(int n) { return ceil_div(n, kBlrB); }
struct BlrSys {
    const void *A;          // complex64, leading dimension lda
    size_t lda;
    int n;
    int *rank;              // [nb][nb] rank of block (I, J), -1: dense
    float2 *U, *V;          // FP32 work terms [nb * nb][kBlrMaxRank][kBlrB]: U[b][l][i], V[b][l][j]
    unsigned *U16, *V16;    // the kept factors as fp16 pairs, same layout
    float *scale;           // [nb * nb][kBlrMaxRank]
};
struct BlrBatch {
    int B;
    int off[kMaxAsm + 1];   // prefix of blocks (one warp each)
    BlrSys sys[kMaxAsm];
};
void blr_batch_finish(BlrBatch &t);
cudaError_t launch_blr_compress(const BlrBatch &t, cudaStream_t st);

// ---------------------------------------------------------------- Krylov engine
// Restarted GMRES of one system as a state machine on the device.  An
// iteration body (one captured graph) runs kSteps Arnoldi steps for every
// system in phase ARNOLDI, then the cycle end for every system in phase
// UPDATE: y = H^{-1} g, x += d = M^{-1} V y, the refinement residual, the
// convergence decision and the restart.  The residual is r = b - A x with
// error-free products after the first cycle (and always for complex128);
// complex64 systems then update it as r -= A d with the plain product: the
// later corrections d are about 1e-5 |x|, so the product's rounding stays
// near 1e-10 |b|.
enum KPhase : int { kPhaseIdle = 0, kPhaseArnoldi = 1, kPhaseUpdate = 2, kPhaseFinished = 3 };
enum KResult : int { kResRunning = 0, kResConverged = 1, kResMaxIter = 2, kResStagnated = 3, kResBreakdown = 4 };

struct KState {
    int phase, k, iters, cycles;
    int result, m, max_iter, n_mv;
    double tol;          // relative residual target
    double floor_rel;    // inner cycle stops at floor_rel * beta (mixed: 3e-4
                         // with the fp16 copy, 1e-5 without)
    double bnorm, beta, prev_beta, thr, res, rel;
};

struct KSys {
    const void *A;          // complex64 or complex128, row-major
    long long lda;
    int n, pc;              // pc: apply Minv
    int nchunk, nvb;        // mv_chunks(n), vec_blocks(n)
    const void *Minv;
    double2 *x, *b, *r, *w, *z, *V;   // V: kMaxRestart + 1 vectors, stride ldv;
                                      // complex64 systems: w, V (and the inner-
                                      // product partials) hold float pairs
    float2 *xh;             // complex64 systems: float copy of the next product's input
    float4 *xf;             // complex64 systems: x as (hi, lo) floats, chunk-permuted
    long long ldv;
    double2 *mvp;           // matvec partials [nchunk][n]
    double2 *dpa, *dpb;     // inner-product partials [kMaxRestart + 1][nvb]
    double *nrmp;           // squared-norm partials [nvb]
    double2 *H, *cs, *sn, *g, *y, *hsum;   // H: (m + 1) x m row-major
    int shared;             // 1: shares A with its neighbours in the table (one
                            // solver's right-hand sides; complex64 only); its
                            // product is one full-row partial (nchunk = 1)
    const void *A16;        // complex64 systems: fp16 copy of A (leading
                            // dimension lda) for the Krylov products, or nullptr
    const float *rs;        // its segment scales (SplitSys::rs)
    int cgs1;               // one classical Gram-Schmidt pass instead of two
    int pcw;                // window correction of the preconditioner (needs pc)
    void *pcy, *pcz;        // its vectors X v and A_w X v: float2 for complex64
                            // systems, double2 for complex128
    int strip;              // rows per item of the TMA product (0: kTmaStrip)
    int blr_nb;             // > 0: the Krylov products read the block low-rank
                            // copy (blr_nb block rows; BlrSys) over A16
    const int *blr_rank;
    const unsigned *blr_U16, *blr_V16;
    const float *blr_scale;
    KState *st;
};

// Systems first .. first + count - 1 of a table share one complex64 matrix.
constexpr int kMaxGroup = 8;   // right-hand sides per shared-matrix product
struct KGroup {
    int first, count;
};

// Systems taking part in one matrix-vector launch and their item offsets;
// rebuilt on the device (k_givens, k_decide) before each launch, so that a
// launch touches only active systems and an empty launch ends at once.
struct KPlan {
    int n;                   // systems in the plan
    int off[kMaxSys + 1];    // prefix sums of their items; off[n] = total
    int sys[kMaxSys];        // their slots in the table
};

struct KTable {
    int B;
    int prec;               // 0: complex128 tiles, 1: complex64 strips
    int vb_total;           // vector blocks of all systems
    int err;                // set when a bounded device wait gave up
    int pcw_any;            // some system applies the window correction
    long long wait_cycles;  // bound of the products' mbarrier waits in clock
                            // cycles (0: the default of about 2 s); a test
                            // sets it low to make a wait run out
    int wait_kinds;         // product kinds (bit k: kind k) the bound applies to
    unsigned mv_ctr[2];     // work queue of the persistent matvec
    KPlan plan[3];          // [0] Krylov product, [1] refinement residual with
                            // error-free products, [2] recursive residual update
    int n_groups;           // shared-matrix groups
    KGroup grp[kMaxSys];
    KPlan gplan[3];         // plans of the shared-matrix products (entries = groups)
    KPlan bplan;            // Krylov products from block low-rank copies (k_mv_blr)
    unsigned gmask[3][kMaxSys];   // per plan entry: members taking part
    const int2 *vb_items;   // (system, block)
    int grp_umma;           // 1: the groups' Krylov products run on the 5th-generation
                            // tensor cores (k_mv_grp_umma; 128-row strips),
                            // 0: on the warp-level ones (k_mv_grp_tc; 32-row strips)
    KSys sys[kMaxSys];
    // TMA tensor maps of the groups' matrices (complex64 rows viewed as
    // 2 n floats; boxes of 32 floats x 128 rows, 128-byte swizzle)
    alignas(64) CUtensorMap gmap[kMaxSys / 2];
};
// The grouped Krylov product on the 5th-generation tensor cores (unless
// BEM_GB300_GROUP_PRODUCT=mma selects the warp-level kernel): TF32 operands,
// so an inner GMRES cycle of a group member stops at 3e-4 of its starting
// residual, like the fp16 copy.
bool group_product_umma();
constexpr int kUmRows = 128;

// Shared-matrix product: items are strips of rows over all columns (32 rows
// for the Krylov product, 16 for the refinement residual), stages of 256
// columns.
constexpr int kGrpRowsInner = 32;
constexpr int kGrpRowsExact = 16;
constexpr int kGrpCols = 256;

// Arnoldi steps per iteration body.
constexpr int kSteps = 8;
// Enqueues one iteration body for the systems of *d_tab (device memory) on
// st.  mv_ev: 2 * (kSteps + 1) events recorded around the matrix-vector
// products (may be nullptr).  prec: 0 complex128, 1 complex64 matrices.
// groups: include the shared-matrix (group) products, for batches that have
// groups; blr: include the block low-rank product (k_mv_blr), for batches
// with systems that have a block low-rank copy; dense: include the Krylov
// product from A or its fp16 copy (k_mv_tma / k_mv64), for batches with
// single systems without one (always for complex128).  Returns the number of
// kernel launches enqueued through *launches_out.
cudaError_t launch_krylov_body(int prec, const KTable *d_tab, cudaEvent_t *mv_ev, cudaStream_t st,
                               int *launches_out, bool groups, bool blr, bool dense);
// complex64 matrices: the product streams row segments with bulk copies
// (TMA) in strips of `strip` rows (a multiple of kTmaRows, chosen per system
// by the tuner; kTmaStrip by default); complex128: tiles of kMvRows rows.
constexpr int kTmaRows = 8;
constexpr int kTmaStrip = 64;
constexpr int kTmaStripMax = 256;
__host__ __device__ inline int mv_items_of(int n, int prec, int strip = kTmaStrip) {
    return ceil_div(n, prec == 0 ? kMvRows : strip) * mv_chunks(n);
}
// Krylov products from the fp16 copy of A: items span two column chunks
// (8 KB row segments, the size the complex64 items move).
__host__ __device__ inline int mv_items16(int n, int strip = kTmaStrip) {
    return ceil_div(n, strip) * ceil_div(mv_chunks(n), 2);
}

// ---------------------------------------------------------------- tuner
// Launch shapes chosen by timing candidates with CUDA events on the first
// call per (device model, size bucket, precision, right-hand sides), kept in
// memory and in a cache file (bem_tune.cu).  Only shapes that leave every
// result bit unchanged are tuned.
struct TuneChoice {
    AsmShape asm_shape;
    int mv_strip = kTmaStrip;   // rows per item of the complex64 product
    bool asm_tuned = false, mv_tuned = false;
    double asm_ms = 0.0, mv_ms = 0.0;   // time of the chosen candidate
};
bool tune_enabled();
int tune_bucket(int n);
TuneChoice tune_lookup(int n, int prec, int n_rhs);
void tune_store_asm(int n, int prec, int n_rhs, AsmShape s, double ms);
void tune_store_mv(int n, int prec, int n_rhs, int strip, double ms);
// One Krylov product (kind 0) of the systems in plan[0] of *d_tab, outside
// any iteration body (the tuner times it).
cudaError_t launch_product(KTable *d_tab, int prec, cudaStream_t st);
// Rebuilds both launch plans of *d_tab from the systems' current phases.
cudaError_t launch_plans(KTable *d_tab, cudaStream_t st);
// Scratch sizes of one system (complex entries).
inline size_t mvp_elems(int n) { return (size_t)mv_chunks(n) * (size_t)n; }
inline size_t xsplit_elems(int n) { return (size_t)mv_chunks(n) * kMvChunk; }
inline size_t dp_elems(int n) { return (size_t)(kMaxRestart + 1) * (size_t)vec_blocks(n); }

}  // namespace bem
