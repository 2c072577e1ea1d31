/* Test infrastructure (oracle only): a plain-C FP64 restatement of the
 * reference NumCalc's traditional-BEM path (Burton-Miller collocation with
 * constant elements).  It is the checker for the CUDA library and the CPU
 * baseline ("port") of the bench; the product never links or calls it.
 *
 * Every function cites the reference routine it restates (paths relative to
 * mesh2hrtf/NumCalc/src/).  Threads: assembly and projection split rows /
 * points over OpenMP threads; results do not depend on the thread count. */
#ifndef BEM_ORACLE_H
#define BEM_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int n_elem;             /* boundary elements (= unknowns), in input order */
    const double *nodes;    /* node coordinates, [n_nodes][3]              */
    const int *conn;        /* [n_elem][4] node indices, -1 past nvert     */
    const int *nvert;       /* 3 (triangle) or 4 (quadrilateral)           */
    const int *bc_type;     /* 0 velocity, 1 pressure, 2 velocity+admittance */
    const double *bc_val;   /* [n_elem][4] complex nodal BC value (zbval0), */
                            /* already in potential units                   */
    const double *adm;      /* [n_elem] complex admittance (zbval1), scaled */
    int sym[3];             /* symmetry plane normal to axis k, coded as the */
                            /* reference holds it after NC_Input.cpp:470-491: */
                            /* 0 none, 1 / 2 symmetric, -1 / -2 antisymmetric */
    double sym_coord[3];    /* plane position on axis k                      */
} or_mesh;

typedef struct {
    double k;               /* wave number                                   */
    double htf;             /* harmonic time factor (+1: e^{-iwt})           */
    double tao;             /* +1 exterior, -1 interior                       */
    int n_point;            /* point sources                                  */
    const double *ps_xyz;   /* [n_point][3]                                  */
    const double *ps_amp;   /* [n_point] complex (zposoc = Q / (i rho w))    */
    int n_plane;            /* plane waves                                   */
    const double *pw_dir;   /* [n_plane][3] unit directions                  */
    const double *pw_amp;   /* [n_plane] complex (zinwav)                    */
} or_freq;

/* Centres, normals (centre + nodes, [n][15]) and areas:
 * NC_ReadMesh, NC_Input.cpp:522-602. */
void or_geometry(const or_mesh *m, double *centers, double *normals, double *areas);

/* Subelements of element j seen from point x: NC_GenerateSubelements,
 * NC_3dFunctions.cpp:575-783.  Returns the count (<= 220) or -1 when the
 * reference would stop with an error. */
int or_subelements(const or_mesh *m, int j, const double x[3], double area,
                   double *xi, double *eta, double *fac, int *order);

/* Rows [row0, row1) of the TBEM system A (row-major, complex, leading
 * dimension n_elem) and the matching right-hand side entries:
 * NC_BuildSystemTBEM / NC_ComputeEntriesForTBEM / NC_AssembleTBEM /
 * NC_SingularIntegration / NC_RegularIntegration / NC_IncidentWaveRHS,
 * NC_EquationSystem.cpp:79-302,1408-1812, with the images of every element
 * in the symmetry planes (NC_ReflectElement / NC_ReflectPointVector,
 * NC_3dFunctions.cpp:181-242,357-452).  Returns 0 or -1 on error. */
int or_assemble(const or_mesh *m, const double *centers, const double *normals,
                const double *areas, const or_freq *f, int row0, int row1,
                double *A, double *rhs, int nthreads);

/* Dense complex LU with partial pivoting, overwriting A; x = A^{-1} b. */
int or_solve_dense(int n, double *A, const double *b, double *x);

/* NumCalc's iterative solver: CGS with right preconditioning and unconjugated
 * inner products, stopped at err_rel < tol (relative to the residual after
 * the first update) or at niter_max (NC_IterativeSolverCGS,
 * NC_CommonFunctions.cpp:1066-1208), on y = A M^-1 x products
 * (NC_MatrixVectorMultiplication case 0, 1211-1245).  precond 0: threshold
 * ILU of scanning degree scan (NC_IncompleteLUDecomposition TBEM branch and
 * NC_IncompleteLUForBack, 1357-1721; it scales the rows of A and b in place);
 * 1: row scaling (NC_ComputeScalingVector, 1322-1354); 2: none.  On
 * iteration failure it runs the reference's dense LU without pivoting
 * (Tfactor_usy / Tfbelim, NC_TypeDefinition.h:543-594).  A and b are
 * overwritten.  stage_s (may be NULL): seconds of preconditioner set-up,
 * iterations, and the final (un)preconditioning or direct solve.  Returns 0,
 * 1 when the direct solver ran, -1 on allocation failure. */
int or_solve_cgs(int n, double *A, double *b, int precond, int scan, int niter_max, double tol, double *x,
                 int *iters, double *rel_err, int nthreads, double *stage_s);

/* Potential and its gradient at points: NC_ContributionTBEM /
 * NC_IntegrationTBEM / NC_ContributionIncidentWaves,
 * NC_PostProcessing.cpp:776-975,1217-1322 (with the element and source
 * images of the symmetry planes).  phi: element potentials
 * (cVpotele), vel: [n][4] complex nodal normal velocities (cVeloele). */
int or_project(const or_mesh *m, const double *centers, const double *normals,
               const double *areas, const or_freq *f, const double *phi,
               const double *vel, int npts, const double *pts, double *pot,
               double *grad, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
