/* bem_gb300.h - C ABI of the GB300 traditional-BEM library.
 *
 * Boundary-element solver for exterior/interior Helmholtz problems in
 * Burton-Miller form with constant (one unknown per element) triangular and
 * quadrilateral elements, the method of Mesh2HRTF's NumCalc when it runs its
 * traditional BEM (methodBEM = 0).  The reference has no library API: its only
 * interface is the NumCalc process.  Each entry point below takes over one
 * phase of NumCalc's per-frequency loop (mesh2hrtf/NumCalc/src/NC_Main.cpp:
 * 370-963); the file:line after each declaration names the reference routine
 * it replaces.  The drop-in NumCalc executable of this project is the main
 * caller; Python tooling binds the same symbols through ctypes.
 *
 * Conventions (as in NumCalc): time factor e^{-i w t} (time_factor = +1) or
 * e^{+i w t} (-1); Green's function e^{i k r}/(4 pi r); unknown = velocity
 * potential phi for velocity/admittance elements and normal velocity for
 * pressure elements; pressure = i rho w phi.  Complex numbers are two
 * doubles (re, im).  All host pointers are read during the call only.
 * Every call returns a bem_status; bem_last_error() gives a message for the
 * calling thread.  One bem_solver_t must not be used by two threads at once.
 */
#ifndef BEM_GB300_H
#define BEM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    BEM_OK = 0,
    BEM_ERR_INVALID = 1,        /* bad argument or unsupported input          */
    BEM_ERR_OUT_OF_HBM = 2,     /* admission refused: footprint above budget   */
    BEM_ERR_NOT_CONVERGED = 3,  /* Krylov solver hit its iteration limit       */
    BEM_ERR_DEVICE_TIMEOUT = 4, /* a bounded device wait gave up               */
    BEM_ERR_CUDA = 5,           /* CUDA runtime error                          */
    BEM_ERR_SUBDIVISION = 6,    /* element subdivision limit exceeded (NumCalc
                                   stops with the same condition)              */
    BEM_ERR_PENDING = 7         /* a served request is not finished yet        */
} bem_status;

typedef enum {
    BEM_PREC_FP64 = 0,   /* FP64 assembly, complex128 matrix, FP64 GMRES        */
    BEM_PREC_MIXED = 1   /* FP32 assembly (FP64 free terms and exact            */
                         /* subdivision decisions), complex64 matrix with an    */
                         /* fp16 Krylov copy, restarted GMRES in FP32 inside an */
                         /* iterative refinement whose residuals reach FP64     */
                         /* accuracy (compensated products)                     */
} bem_precision;

typedef struct bem_mesh_s *bem_mesh_t;
typedef struct bem_solver_s *bem_solver_t;

/* Boundary mesh.  Element order defines the unknown order (NumCalc's jelist,
 * NC_Addresses.cpp:179-184).  centers/normals/areas may be NULL, in which case
 * they are computed with NumCalc's formulas (NC_Input.cpp:522-602); the
 * drop-in passes the values its parser computed so that both agree bit for
 * bit. */
typedef struct {
    int32_t n_elem;
    int32_t n_nodes;
    const double *nodes;     /* [n_nodes][3]                                  */
    const int32_t *conn;     /* [n_elem][4] node indices, -1 past nvert       */
    const int32_t *nvert;    /* [n_elem] 3 or 4                               */
    const double *centers;   /* [n_elem][3] or NULL                           */
    const double *normals;   /* [n_elem][3] unit normal at the centre or NULL */
    const double *areas;     /* [n_elem] or NULL                              */
    /* Symmetry planes (NC.inp SYMMETRY block, NC_Input.cpp:459-494): per axis
     * the NC.inp code (0 none, 1 symmetric, 2 antisymmetric, 3 / 4 hard /
     * soft reflecting, which the traditional BEM treats as 1 / 2) and the
     * plane's position on that axis.  The mesh is the part on one side of
     * the planes; every element is integrated with its 1, 2, 4 or 8 images
     * (NC_ReflectElement, NC_3dFunctions.cpp:357-452) and incident waves
     * with theirs.  All zero: no planes. */
    int32_t sym_planes[3];
    double sym_coords[3];
} bem_mesh_desc;

/* Per-frequency data: NumCalc's state after NC_UpdateFreqCurves
 * (NC_EquationSystem.cpp:1815-1961). */
typedef struct {
    double wave_number;        /* k = 2 pi f / c                               */
    double time_factor;        /* +1 or -1                                     */
    double tao;                /* +1 exterior, -1 interior problem             */
    const int32_t *bc_type;    /* [n_elem] 0 velocity, 1 pressure,
                                  2 velocity + surface admittance; NULL = 0    */
    const double *bc_value;    /* [n_elem][4] complex nodal values (zbval0),
                                  potential units; NULL = 0                    */
    const double *admittance;  /* [n_elem] complex (zbval1, already scaled by
                                  i k time_factor); NULL = 0                   */
    int32_t n_point;           /* point sources                                */
    const double *point_xyz;   /* [n_point][3]                                 */
    const double *point_amp;   /* [n_point] complex: NC.inp amplitude/(i rho w)*/
    int32_t n_plane;           /* plane waves                                  */
    const double *plane_dir;   /* [n_plane][3] unit direction                  */
    const double *plane_amp;   /* [n_plane] complex: amplitude/(i rho w)       */
} bem_frequency_desc;

typedef struct {
    int32_t precision;         /* bem_precision                                */
    int32_t restart;           /* GMRES restart length (0 = default 60,
                                  at most 63)                                  */
    int32_t max_iter;          /* total inner iterations (0 = default 1000)    */
    double tol;                /* relative residual target (0 = 1e-9)          */
    double hbm_budget_bytes;   /* admission budget for this solver (0 = all
                                  free device memory minus a reserve)          */
    int32_t no_precond;        /* 0 (default): block-Jacobi inverse X of the
                                  128-unknown diagonal blocks with one
                                  correction step over 1024-unknown diagonal
                                  windows A_w, M = X (2 I - A_w X);
                                  1: none; 2: block-Jacobi only (M = X);
                                  3: NumCalc's scaling preconditioner, the
                                  diagonal d_i = sqrt(N / sum_j |a_ij|^2)
                                  on the right (NC_ComputeScalingVector,
                                  NC_CommonFunctions.cpp:1322-1351)           */
    int32_t n_rhs;             /* right-hand sides the solver can hold for
                                  bem_solve_multi (0 or 1: one; at most 16)    */
    int32_t complex64_krylov;  /* mixed precision with one right-hand side:
                                  0 (default) the Krylov products read an fp16
                                  copy of A (row-scaled; 4 bytes per entry,
                                  +50 % matrix memory) and the refinement
                                  residuals the complex64 matrix; 1 every
                                  product reads the complex64 matrix; 2 the
                                  Krylov products read a block low-rank copy
                                  over the fp16 one (off-diagonal 256 x 256
                                  blocks compressed by adaptive cross
                                  approximation, checked to 2e-4 with random
                                  probes, fp16 factors; the other blocks from
                                  the fp16 copy; about +100 % matrix memory):
                                  fewer bytes per product, but the compression
                                  costs about as much as 10-20 products, so it
                                  pays off in batches and long solves        */
} bem_solver_params;

typedef struct {
    int32_t iterations;        /* Krylov iterations (matrix-vector products)   */
    int32_t restarts;          /* outer cycles (explicit residuals)            */
    double rel_residual;       /* final ||b - A x|| / ||b||                    */
    double assemble_ms;        /* device time of the last bem_assemble         */
    double solve_ms;           /* device time of the last bem_solve            */
    double project_ms;         /* device time of the last bem_project          */
    int64_t n_near_pairs;      /* element pairs that needed subdivision        */
    double matvec_ms;          /* device time of the matrix-vector products of
                                  the last bem_solve (inner and residual)      */
    int32_t n_matvec;          /* number of those products                     */
} bem_solve_info;

/* Library / device ------------------------------------------------------- */
const char *bem_last_error(void);
const char *bem_version(void);
/* Number of CUDA kernels this library has launched in this process (all
 * devices).  Diagnostic with no counterpart in the reference. */
int64_t bem_kernel_launches(void);
/* Measured issue rates of a device, in operations per second over the whole
 * device: rates[0] FP32 FMA, rates[1] special-function approximations
 * (sin / cos / rsqrt), rates[2] FP64 FMA.  Micro-kernels of independent
 * dependency chains in every lane, timed with CUDA events (best of three);
 * they are the denominators of the compute-bound stages' rooflines.
 * Diagnostic with no counterpart in the reference.  Sets the device. */
bem_status bem_measure_issue_peaks(int32_t device, double *rates);
/* The launch shapes the tuner holds for a system size, precision and
 * right-hand-side count on the current device, as a JSON object written to
 * buf (len bytes): the assembly's persistent grids (k_far / k_near resident
 * blocks per SM), the complex64 product's strip height (rows per work item),
 * whether each was tuned, the time of the chosen candidate, and the
 * defaults.  The library times the candidates with CUDA events on the first
 * assembly and the first solve of each (device model, size bucket,
 * precision, right-hand sides), keeps the fastest in memory and appends it
 * to a cache file ($BEM_GB300_TUNE_CACHE, else
 * $XDG_CACHE_HOME/mesh2hrtf_gb300/tune.txt, else
 * ~/.cache/mesh2hrtf_gb300/tune.txt); BEM_GB300_TUNE=0 keeps the defaults.
 * Only shapes that leave every result bit unchanged are tuned.  No
 * counterpart in the reference. */
bem_status bem_tune_info(int32_t n_elem, int32_t precision, int32_t n_rhs, char *buf, int32_t len);
/* Select the CUDA device for this thread's subsequent calls. */
bem_status bem_set_device(int32_t device);
/* Bytes a solver for n_elem unknowns holds on the device (matrix, Krylov
 * basis, preconditioner, work vectors) at the given precision and restart
 * length, with the default Krylov copy: the HBM
 * admission footprint (NumCalc's host RAM estimate, NC_Main.cpp:524-541,
 * counts (N + N^2) * 16 bytes for the same data).  The block low-rank copy
 * (complex64_krylov = 2) adds about 295 KB per block of 256 x 256 unknowns,
 * ceil(N / 256)^2 blocks (1.9 GB at N = 20480); bem_solver_create checks
 * the whole footprint against the budget. */
double bem_footprint_bytes(int32_t n_elem, int32_t precision, int32_t restart);
/* The same for a solver holding n_rhs right-hand sides (bem_solve_multi). */
double bem_footprint_multi(int32_t n_elem, int32_t precision, int32_t restart, int32_t n_rhs);
/* Bytes a mesh of n_elem elements with n_sym_planes symmetry planes holds on
 * the device: element tables, symmetry images and the near-pair list (48
 * pairs per element and image, grown to the exact count when the geometry
 * needs more).  Host arithmetic only, no device needed. */
double bem_mesh_footprint_bytes(int32_t n_elem, int32_t n_sym_planes);
/* Free and total device memory of a device (cudaMemGetInfo; creates the
 * device's context in the calling process).  free_bytes counts the blocks
 * the library keeps cached for reuse (see bem_release_cached_memory). */
bem_status bem_device_memory(int32_t device, double *free_bytes, double *total_bytes);
/* Meshes, solvers and point buffers release their device memory into a
 * per-device cache that the next creation of about the same size reuses
 * (cudaFree of GB-sized blocks synchronizes the device and takes
 * milliseconds).  This returns the cached blocks to the driver.  Environment
 * BEM_GB300_CACHE=0 turns the cache off. */
bem_status bem_release_cached_memory(void);

/* Mesh: upload and precompute element tables.
 * Replaces NC_ReadMesh's geometry part (NC_Input.cpp:522-602) and the per-pair
 * element gather NC_ComputeElementData (NC_3dFunctions.cpp:245-354). */
bem_status bem_mesh_create(const bem_mesh_desc *desc, bem_mesh_t *out);
bem_status bem_mesh_destroy(bem_mesh_t mesh);

/* Solver workspace on the device (matrix + Krylov state), admitted against
 * params->hbm_budget_bytes.  Replaces the per-frequency allocations of
 * NC_Main.cpp:744-757 and NC_Addresses.cpp:236-238. */
bem_status bem_solver_create(bem_mesh_t mesh, const bem_solver_params *params,
                             bem_solver_t *out);
bem_status bem_solver_destroy(bem_solver_t solver);
/* Change the tolerance and the iteration limit of an existing solver (the
 * precision and restart length are fixed at creation); fields <= 0 keep
 * their value.  NumCalc's -nitermax option (NC_Main.cpp:171-175) sets the
 * CGS limit the same way. */
bem_status bem_solver_set_params(bem_solver_t solver, const bem_solver_params *params);

/* Assemble A and b for one frequency.
 * Replaces NC_SetupEquationSystem / NC_BuildSystemTBEM /
 * NC_ComputeEntriesForTBEM / NC_AssembleTBEM / NC_SingularIntegration /
 * NC_RegularIntegration / NC_IncidentWaveRHS
 * (NC_EquationSystem.cpp:79-302,1408-1812) and NC_GenerateSubelements
 * (NC_3dFunctions.cpp:575-783). */
bem_status bem_assemble(bem_solver_t solver, const bem_frequency_desc *freq);

/* Solve A x = b.  Replaces NC_IterativeSolverCGS with its preconditioners
 * and direct fallback (NC_CommonFunctions.cpp:1066-1208,1322-1721) by a
 * restarted GMRES (see bem_precision). */
bem_status bem_solve(bem_solver_t solver, bem_solve_info *info);

/* Solve A x = b directly: LU factorisation without pivoting in place, then
 * forward and back substitution, for every right-hand side the solver holds.
 * Replaces Tfactor_usy / Tfbelim (NC_TypeDefinition.h:543-594), which NumCalc
 * runs for ISOLVER 4 (NC_Main.cpp:833-866) and after a failed CGS
 * (NC_CommonFunctions.cpp:1181-1191).  The factorisation runs in the matrix's
 * precision (complex128 for BEM_PREC_FP64, complex64 for BEM_PREC_MIXED), the
 * substitutions in FP64.  A holds the factors afterwards: bem_solve and a
 * second bem_solve_direct need a new bem_assemble, and bem_get_system returns
 * the factors (L unit lower, U upper).  info gets no iterations and a
 * residual of 0 (not computed); a zero pivot gives BEM_ERR_INVALID. */
bem_status bem_solve_direct(bem_solver_t solver, bem_solve_info *info);

/* The block low-rank Krylov copy of a solver created with
 * complex64_krylov = 2, as of its last assembly: blocks per block row,
 * blocks read from the fp16 copy (the diagonal ones and those whose cross
 * approximation needed more than 48 terms or failed the probe check), the
 * mean rank of the compressed ones, and the bytes one Krylov product moves
 * (fp16 factors and scales, fp16 dense blocks, the input vector and row
 * scales per item, and the partial sums it writes).  Synchronous.  A solver
 * without that copy gives BEM_ERR_INVALID.  No counterpart in NumCalc. */
bem_status bem_krylov_copy_info(bem_solver_t solver, int32_t *blocks_per_row, int32_t *dense_blocks,
                                double *mean_rank, double *bytes_per_product);

/* Copy the solution (complex, n_elem) to host memory. */
bem_status bem_get_solution(bem_solver_t solver, double *x_host);

/* Copy the assembled matrix rows [row0, row1) (complex, row-major, n_elem
 * columns, converted to FP64) and the right-hand side to host memory; NULL
 * skips either.  For tests and diagnostics. */
bem_status bem_get_system(bem_solver_t solver, int32_t row0, int32_t row1,
                          double *a_host, double *b_host);

/* Potential and its gradient at n_pts field points (host arrays), from the
 * boundary data of the last solve plus the incident field.
 * Replaces the TBEM branch of NC_WriteResultsEvaluationGrid with
 * NC_ContributionTBEM / NC_IntegrationTBEM / NC_ContributionIncidentWaves
 * (NC_PostProcessing.cpp:581-773,776-975,1217-1322).  pot_out: [n_pts]
 * complex; grad_out: [n_pts][3] complex (may be NULL). */
bem_status bem_project(bem_solver_t solver, int32_t n_pts, const double *pts,
                       double *pot_out, double *grad_out);

/* Field projection that allocates nothing.
 *
 * Same result as bem_project, but points and outputs are device pointers the
 * caller owns and the call makes no device allocation (no cudaMalloc,
 * cudaFree or allocating library routine): its scratch lives in a fixed
 * device array inside the library.  It is meant for callers that must not
 * allocate once they are running, for example a real-time renderer or audio
 * plug-in host that evaluates the solved field at new listener positions on
 * every processing block (an allocation there can block or synchronize the
 * device), or code that manages all device memory through its own pool.
 * No counterpart in the reference (NumCalc only projects onto the grids of
 * NC.inp, NC_PostProcessing.cpp:581-773).
 *
 * Limits and rules:
 *  - at most BEM_STATIC_MAX_ELEMENTS boundary elements (larger solvers get
 *    BEM_ERR_INVALID); the scratch array (about 12.4 MB: 4.1 MB of element
 *    data plus 8 MB of partial sums) is held on every device that loads the
 *    library until the process exits;
 *  - the first call on a device looks up the array's device address;
 *  - the call is synchronous: it runs on `stream` (a cudaStream_t, NULL for
 *    the legacy default stream), reads the status word back and returns
 *    after the stream has finished, so it cannot be recorded into a CUDA
 *    graph;
 *  - the calling thread's current device, the stream's device and the
 *    solver's device must be the same (else BEM_ERR_INVALID);
 *  - all calls share the one array, so calls that overlap on the GPU (other
 *    streams, other threads) race: serialize them.  The call reads the
 *    solver's solution and mesh tables and writes none of its buffers, but
 *    it must not overlap a bem_assemble or bem_solve of the same solver;
 *  - with many points and elements the partial sums take wider element
 *    slices than bem_project's (a different FP32 summation order in mixed
 *    precision, same quadrature);
 *  - pts_dev [n_pts][3] FP64, pot_dev [n_pts] complex, grad_dev [n_pts][3]
 *    complex or NULL, all device memory. */
#define BEM_STATIC_MAX_ELEMENTS 32768
bem_status bem_project_static(bem_solver_t solver, int32_t n_pts, const double *pts_dev,
                              double *pot_dev, double *grad_dev, void *stream);

/* One complete frequency step through host buffers: assemble, solve, copy
 * the unknowns to x_out (may be NULL) and project onto n_pts points.
 * The sequence NC_Main.cpp:744-907 runs per frequency. */
bem_status bem_solve_frequency(bem_solver_t solver, const bem_frequency_desc *freq,
                               int32_t n_pts, const double *pts, double *x_out,
                               double *pot_out, double *grad_out,
                               bem_solve_info *info);

/* Several right-hand sides on one matrix: one assembly of A, one
 * preconditioner, then n_rhs GMRES iterations in lockstep whose products
 * share each read of A, and one projection pass.  Right-hand side r takes the
 * sources and prescribed boundary values of freqs[r]; the wave number,
 * time factor, tao, boundary-condition types and admittances (which define
 * the matrix) are those of freqs[0].  NumCalc sums all sources of a project
 * into one right-hand side (NC_IncidentWaveRHS, NC_EquationSystem.cpp:
 * 1731-1812); Mesh2HRTF runs one project per source (the ears), i.e. one
 * NumCalc per right-hand side.  Needs a solver created with n_rhs >= the
 * count.  x_out[r] (n_elem complex), pot_out[r] ([n_pts] complex) and
 * grad_out[r] ([n_pts][3] complex) may be NULL arrays or hold NULLs;
 * infos[r] (may be NULL) gets right-hand side r's iterations and residual. */
bem_status bem_solve_multi(bem_solver_t solver, int32_t n_rhs, const bem_frequency_desc *freqs,
                           int32_t n_pts, const double *pts, double *const *x_out,
                           double *const *pot_out, double *const *grad_out,
                           bem_solve_info *infos);

/* Several frequency steps solved together: count (solver, frequency)
 * instances, each solver with its own mesh (meshes of different sizes mix
 * freely; a solver may appear once).  The assembly of all instances runs as
 * one persistent launch, their GMRES iterations run in lockstep inside one
 * captured iteration body, and their projections run as one launch.  Each
 * instance's result is the one bem_solve_frequency gives for it alone.
 * NumCalc runs such steps as separate processes (manage_numcalc.py:376-378);
 * no counterpart inside the reference.
 *
 * Arrays are indexed by instance; n_pts, pts, x_out, pot_out, grad_out,
 * infos and statuses may be NULL, and entries of the pointer arrays may be
 * NULL where nothing is wanted.  infos[i] holds instance i's iterations and
 * residual; its times are those of the whole batch.  statuses[i] is the
 * instance's own status; the return value is BEM_OK or the first failing
 * instance's status.  Runs on a stream owned by the calling thread. */
bem_status bem_solve_batch(int32_t count, const bem_solver_t *solvers,
                           const bem_frequency_desc *freqs, const int32_t *n_pts,
                           const double *const *pts, double *const *x_out,
                           double *const *pot_out, double *const *grad_out,
                           bem_solve_info *infos, bem_status *statuses);

/* Serving ----------------------------------------------------------------
 * A server takes solve requests ((mesh, frequency, evaluation points)) as
 * they arrive and runs them with continuous batching: a request is admitted
 * when its footprint (bem_footprint_bytes plus its points) fits the free part
 * of the server's device-memory budget and an iteration slot is free; its
 * assembly runs on a second stream while the admitted requests iterate; it
 * joins the batched GMRES at the next iteration body and leaves it when it
 * has converged, after which it is projected and its memory is returned.
 * Requests are admitted in arrival order.  A request's result is the one
 * bem_solve_frequency gives for it alone.  NumCalc has no counterpart: its
 * steps run as processes that manage_numcalc starts while host RAM allows
 * (manage_numcalc.py:284-385). */
typedef struct bem_server_s *bem_server_t;

typedef struct {
    int32_t precision;         /* bem_precision of every request               */
    double hbm_budget_bytes;   /* device memory reserved for the requests
                                  (0 = free memory minus 1 GB)                 */
    int32_t max_active;        /* requests iterating together (0 = 128, the
                                  most)                                        */
    int32_t restart;           /* as in bem_solver_params; 0 = defaults        */
    int32_t max_iter;
    double tol;
    int32_t device;            /* CUDA device of the server                    */
} bem_server_params;

typedef struct {
    double queued_ms;          /* submit -> admitted                            */
    double latency_ms;         /* submit -> results ready                       */
    bem_solve_info solve;      /* iterations and residual of the request; the
                                  stage times are those of the launches it took
                                  part in                                       */
} bem_request_info;

/* Reserves the budget on the device and starts the server's worker thread. */
bem_status bem_server_create(const bem_server_params *params, bem_server_t *out);
/* Queue one request; freq, its arrays and pts [n_pts][3] are copied.  The
 * mesh must stay alive until the request has been waited for.  A request
 * whose footprint exceeds the whole budget gets BEM_ERR_OUT_OF_HBM here. */
bem_status bem_server_submit(bem_server_t server, bem_mesh_t mesh, const bem_frequency_desc *freq,
                             int32_t n_pts, const double *pts, uint64_t *ticket);
/* Wait up to timeout_s seconds (< 0: no limit) for a request; copy its
 * unknowns (n_elem complex, may be NULL), potentials [n_pts] and gradients
 * [n_pts][3] (may be NULL) and release the ticket.  Returns the request's own
 * status, or BEM_ERR_PENDING (ticket kept) if it has not finished in time. */
bem_status bem_server_wait(bem_server_t server, uint64_t ticket, double timeout_s, double *x_out,
                           double *pot_out, double *grad_out, bem_request_info *info);
/* Finish the requests already admitted, drop the queued ones, stop. */
bem_status bem_server_destroy(bem_server_t server);

#ifdef __cplusplus
}
#endif
#endif /* BEM_GB300_H */
