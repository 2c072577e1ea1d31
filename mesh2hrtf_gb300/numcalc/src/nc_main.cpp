// nc_main.cpp - the drop-in NumCalc executable.
//
// Same command line, working-directory contract and output files as the
// reference NumCalc (mesh2hrtf/NumCalc/src/NC_Main.cpp:137-281 and the
// frequency loop 284-1048): reads ./NC.inp and the mesh files it lists,
// writes NC.out / NC<i>-<j>.out / NCfrom<i>.out / NCuntil<j>.out,
// be.out/be.<step>/{pBoundary,vBoundary,pEvalGrid,vEvalGrid} and, with
// -estimate_ram, Memory.txt.  Every frequency step is solved on the GPU
// through the C ABI of include/bem_gb300.h as a dense (traditional) BEM,
// whatever method NC.inp selects.
//
// Environment: NUMCALC_GB300_PRECISION = mixed (default) | fp64,
//              NUMCALC_GB300_DEVICE = CUDA device index (default 0),
//              NUMCALC_GB300_WAIT_S = seconds to wait for device memory when
//              other NumCalc processes hold it (default 3600),
//              NUMCALC_GB300_NPY = 1: every result file is also written as
//              <name>.npy (complex128, the printed values at full precision,
//              in the text file's row order) for post-processing without the
//              7-digit text round trip (mesh2hrtf_gb300/output2hrtf.py).
#include <sys/stat.h>
#include <unistd.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <iomanip>
#include <iostream>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "bem_gb300.h"
#include "nc_fmm_plan.h"
#include "nc_project.h"

using nc::cd;

namespace {

const mode_t kDirMode = S_IRUSR | S_IWUSR | S_IXUSR | S_IRGRP | S_IWGRP | S_IXGRP | S_IROTH | S_IXOTH;
// Device memory a CUDA context of this process takes (MemoryGPU.txt).
constexpr double kContextBytes = 0.6e9;

void stamp(std::ostream &o, const char *what, const tm *d) {
    o << what << d->tm_mday << "/" << d->tm_mon + 1 << "/" << d->tm_year + 1900 << " " << d->tm_hour << ":"
      << d->tm_min << ":" << d->tm_sec;
}

// mul_i of NC_TypeDefinition.h: z * (i y)
cd mul_i(cd z, double y) { return cd(-z.imag() * y, z.real() * y); }

struct Gpu {
    bem_mesh_t mesh = nullptr;
    bem_solver_t solver = nullptr;
    ~Gpu() {
        if (solver) bem_solver_destroy(solver);
        if (mesh) bem_mesh_destroy(mesh);
    }
};

[[noreturn]] void gpu_fail(std::ofstream &out, const char *what, bem_status st) {
    std::cout << what << ": " << bem_last_error() << " (status " << (int)st << ")" << std::endl;
    out << what << ": " << bem_last_error() << " (status " << (int)st << ")" << std::endl;
    std::exit(1);
}

// complex128 array as a .npy file (format 1.0, little endian, C order)
void write_npy(const std::string &path, const std::vector<cd> &v, const std::vector<size_t> &shape) {
    if (!std::getenv("NUMCALC_GB300_NPY")) return;
    std::string hdr = "{'descr': '<c16', 'fortran_order': False, 'shape': (";
    for (size_t k = 0; k < shape.size(); ++k) hdr += std::to_string(shape[k]) + (shape.size() == 1 ? "," : k + 1 < shape.size() ? ", " : "");
    hdr += "), }";
    const size_t total = 10 + hdr.size() + 1;
    hdr.append((64 - total % 64) % 64, ' ');
    hdr += '\n';
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) throw nc::NcExit{"Can not open the file " + path, 1};
    const unsigned char magic[8] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0};
    const uint16_t hl = (uint16_t)hdr.size();
    const unsigned char len[2] = {(unsigned char)(hl & 0xff), (unsigned char)(hl >> 8)};
    std::fwrite(magic, 1, 8, f);
    std::fwrite(len, 1, 2, f);
    std::fwrite(hdr.data(), 1, hdr.size(), f);
    std::fwrite(v.data(), sizeof(cd), v.size(), f);
    std::fclose(f);
}

// pBoundary / vBoundary (NC_WriteResultsObjectMesh, NC_PostProcessing.cpp:
// 367-578): element potentials and velocities at the collocation points.
void write_boundary(const nc::Project &p, const nc::FreqState &fs, const std::vector<cd> &x,
                    const std::string &dir) {
    const int NE = p.n_elem;
    std::vector<cd> pot(NE), vel(NE);
    std::vector<int> dof(NE, -1);
    int d = 0;
    for (int e = 0; e < NE; ++e)
        if (p.elem_prop[e] != 2) dof[e] = d++;
    for (int e = 0; e < NE; ++e) {
        if (p.elem_prop[e] == 2) continue;
        const cd xe = x[dof[e]];
        if (p.ibval[e] == 1) {
            pot[e] = fs.zbval0[4 * (size_t)e];
            vel[e] = xe;
        } else {
            pot[e] = xe;
            vel[e] = fs.zbval0[4 * (size_t)e];
            if (p.ibval[e] == 2) vel[e] -= (pot[e] * fs.zbval1[e]) * p.tao;
        }
    }
    std::vector<cd> np_p, np_v;   // the printed values, for write_npy
    FILE *fp = std::fopen((dir + "/pBoundary").c_str(), "w");
    FILE *fv = std::fopen((dir + "/vBoundary").c_str(), "w");
    if (!fp || !fv) throw nc::NcExit{"Can not open the file " + dir + "/pBoundary", 1};
    std::fprintf(fp, "%s\n", p.version.c_str());
    std::fprintf(fv, "%s\n", p.version.c_str());
    std::fprintf(fp, "%5d\n", p.n_groups);
    std::fprintf(fv, "%5d\n", p.n_groups);
    for (int g = 0; g < p.n_groups; ++g) {
        bool has_be = false;
        for (int e = 0; e < NE && !has_be; ++e)
            if (p.elem_prop[e] != 2 && p.elem_group[e] == p.group_index[g]) has_be = true;
        if (!has_be) continue;
        std::fprintf(fp, "%5d %5d\n", p.group_index[g], p.group_count[g]);
        std::fprintf(fv, "%5d %5d\n", p.group_index[g], p.group_count[g]);
        for (int e = 0; e < NE; ++e) {
            if (p.elem_prop[e] == 2 || p.elem_group[e] != p.group_index[g]) continue;
            const cd pr = mul_i(pot[e], fs.rpfact);
            std::fprintf(fp, "%5d % E % E\n", p.elem_ext[e], pr.real(), pr.imag());
            std::fprintf(fv, "%5d % E % E\n", p.elem_ext[e], vel[e].real(), vel[e].imag());
            np_p.push_back(pr);
            np_v.push_back(vel[e]);
        }
    }
    std::fclose(fp);
    std::fclose(fv);
    write_npy(dir + "/pBoundary.npy", np_p, {np_p.size()});
    write_npy(dir + "/vBoundary.npy", np_v, {np_v.size()});
}

// pEvalGrid / vEvalGrid (NC_WriteResultsEvaluationGrid,
// NC_PostProcessing.cpp:581-773).
void write_eval(const nc::Project &p, const nc::FreqState &fs, const std::vector<int> &ev_nodes,
                const std::vector<cd> &pot, const std::vector<cd> &grad, const std::string &dir) {
    FILE *fp = std::fopen((dir + "/pEvalGrid").c_str(), "w");
    FILE *fv = std::fopen((dir + "/vEvalGrid").c_str(), "w");
    if (!fp || !fv) throw nc::NcExit{"Can not open the file " + dir + "/pEvalGrid", 1};
    std::fprintf(fp, "%s\n", p.version.c_str());
    std::fprintf(fv, "%s\n", p.version.c_str());
    int group = -1;
    for (int e = 0; e < p.n_elem; ++e)
        if (p.elem_prop[e] == 2) { group = p.elem_group[e]; break; }
    const int m = (int)ev_nodes.size();
    const int ngrp = m > 0 ? 1 : 0;
    std::fprintf(fv, "%5d\n", ngrp);
    if (m > 0) std::fprintf(fv, "%5d %5d\n", group, m);
    for (int i = 0; i < m; ++i) {
        const cd *g = &grad[3 * (size_t)i];
        std::fprintf(fv, "%5d %E %E %E %E %E %E\n", p.node_ext[ev_nodes[i]], g[0].real(), g[0].imag(), g[1].real(),
                     g[1].imag(), g[2].real(), g[2].imag());
    }
    std::fprintf(fp, "%5d\n", ngrp);
    if (m > 0) std::fprintf(fp, "%5d %5d\n", group, m);
    std::vector<cd> np_p(m);
    for (int i = 0; i < m; ++i) {
        const cd pr = mul_i(pot[i], fs.rpfact);
        std::fprintf(fp, "%5d % E % E\n", p.node_ext[ev_nodes[i]], pr.real(), pr.imag());
        np_p[i] = pr;
    }
    std::fclose(fp);
    std::fclose(fv);
    write_npy(dir + "/pEvalGrid.npy", np_p, {(size_t)m});
    write_npy(dir + "/vEvalGrid.npy", std::vector<cd>(grad.begin(), grad.begin() + 3 * (size_t)m), {(size_t)m, 3});
}

int run(int istart, int iend, bool estimate_ram, bool check_normals, int nitermax, bool nitermax_given,
        std::ofstream &out) {
    time_t ltim[7];
    time_t lti_eqa = 0, lti_sol = 0, lti_pos = 0;
    std::ofstream est, est_gpu;
    if (estimate_ram) {
        est.open("Memory.txt");
        // the same steps with this build's device memory per process, for
        // GPU-aware scheduling (mesh2hrtf_gb300/manage_numcalc.py)
        est_gpu.open("MemoryGPU.txt");
    }
    time(&ltim[0]);
    FILE *inp = std::fopen("NC.inp", "r");
    if (!inp) throw nc::NcExit{"No input file found!", 1};
    out << "\n\n>> G E N E R A L   P A R A M E T E R S <<\n" << std::endl;
    std::cout << "3D analysis" << std::endl;
    out << "\n3D analysis" << std::endl;
    nc::Project p;
    nc::read_project(inp, out, check_normals, p);
    std::fclose(inp);
    time(&ltim[1]);
    if (const char *dump = std::getenv("NUMCALC_GB300_DUMP_TABLES")) {
        // parse-only mode for parser parity checks: tables in the record
        // format of the reference dump harness, then stop
        nc::dump_tables(p, dump);
        return 0;
    }
    time(&ltim[2]);

    // boundary mesh and evaluation points for the device
    const int NE = p.n_elem;
    std::vector<int> be;
    for (int e = 0; e < NE; ++e)
        if (p.elem_prop[e] != 2) be.push_back(e);
    const int N = (int)be.size();
    std::vector<int32_t> conn(4 * (size_t)N, -1), nvert(N), bct(N);
    std::vector<double> cen(3 * (size_t)N), nor(3 * (size_t)N), area(N);
    for (int d = 0; d < N; ++d) {
        const int e = be[d];
        nvert[d] = p.elem_nv[e];
        for (int a = 0; a < p.elem_nv[e]; ++a) conn[4 * (size_t)d + a] = p.elem_conn[4 * (size_t)e + a];
        for (int k = 0; k < 3; ++k) {
            cen[3 * (size_t)d + k] = p.centel[3 * (size_t)e + k];
            nor[3 * (size_t)d + k] = p.elenor[15 * (size_t)e + k];
        }
        area[d] = p.areael[e];
        bct[d] = p.ibval[e];
    }
    std::vector<int> ev_nodes;
    std::vector<double> ev_xyz;
    for (int i = 0; i < p.n_nodes; ++i)
        if (p.node_class[i] == -1) {
            ev_nodes.push_back(i);
            for (int k = 0; k < 3; ++k) ev_xyz.push_back(p.node_xyz[3 * (size_t)i + k]);
        }

    Gpu gpu;
    const char *prec_env = std::getenv("NUMCALC_GB300_PRECISION");
    const int prec = (prec_env && std::string(prec_env) == "fp64") ? BEM_PREC_FP64 : BEM_PREC_MIXED;
    if (!estimate_ram) {
        const char *dev_env = std::getenv("NUMCALC_GB300_DEVICE");
        bem_status st = bem_set_device(dev_env ? std::atoi(dev_env) : 0);
        if (st != BEM_OK) gpu_fail(out, "CUDA device", st);
        bem_mesh_desc md{N, p.n_nodes, p.node_xyz.data(), conn.data(), nvert.data(), cen.data(), nor.data(), area.data(),
                         {0, 0, 0}, {0.0, 0.0, 0.0}};
        // symmetry planes back to their NC.inp codes (the parser holds the
        // reference's internal 1 / -1 / 2 / -2, NC_Input.cpp:474-487)
        for (int k = 0; k < 3 && p.n_sym > 0; ++k) {
            const int c = p.sym_planes[k];
            md.sym_planes[k] = c == 1 ? 1 : c == -1 ? 2 : c == 2 ? 3 : c == -2 ? 4 : 0;
            md.sym_coords[k] = p.sym_coords[k];
        }
        st = bem_mesh_create(&md, &gpu.mesh);
        if (st != BEM_OK) gpu_fail(out, "mesh upload", st);
        bem_solver_params sp{};
        sp.precision = prec;
        sp.tol = 1e-9;   // ErroIterSols, NC_CommonFunctions.cpp:39
        // NC.inp's preconditioner (Main Parameters II, token 4): the
        // incomplete LU (0, any scanning degree) is stood in for by the
        // block-Jacobi preconditioner with its window correction; scaling
        // (1) and none (2) are NumCalc's own
        sp.no_precond = p.precond == 1 ? 3 : p.precond == 2 ? 1 : 0;
        // HBM admission: wait while other NumCalc processes hold the memory
        const char *wait_env = std::getenv("NUMCALC_GB300_WAIT_S");
        const double wait_s = wait_env ? std::atof(wait_env) : 3600.0;
        auto t0 = std::chrono::steady_clock::now();
        while ((st = bem_solver_create(gpu.mesh, &sp, &gpu.solver)) == BEM_ERR_OUT_OF_HBM) {
            const double waited = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            if (waited > wait_s) break;
            std::this_thread::sleep_for(std::chrono::seconds(2));
        }
        if (st != BEM_OK) gpu_fail(out, "solver allocation", st);
    }

    if (iend > 0 && iend > p.n_freq) iend = p.n_freq;
    if (iend == 0) iend = p.n_freq;
    if (istart > 0) istart--;
    std::vector<cd> x(N), pot(ev_nodes.size()), grad(3 * ev_nodes.size());
    // -estimate_ram of an SL-/ML-FMM project reports the reference's FMM
    // estimate
    std::unique_ptr<nc::FmmPlan> fmm;
    if (estimate_ram && p.method_bem != 0) fmm.reset(new nc::FmmPlan(p));
    for (int step = istart; step < iend; ++step) {
        time(&ltim[3]);
        const double f = p.freqs[step];
        std::cout << "\nStep " << step + 1 << ", Frequency = " << f << " Hz" << std::endl;
        out << "\n\n\n>> S T E P   N U M B E R   A N D   F R E Q U E N C Y <<\n" << std::endl;
        out << "Step " << step + 1 << ", Frequency = " << f << " Hz" << std::endl;
        if (step == istart && !fmm) {
            // NC_DeclareArrays / NC_FrequencyInformations for a TBEM step
            const int ncomp = (int)((unsigned)N * (unsigned)N);
            for (std::ostream *o : {(std::ostream *)&std::cout, (std::ostream *)&out}) {
                *o << "\nTraditional BEM" << std::endl;
                *o << "\nNumber of equations = " << N << std::endl;
                *o << "Number of entries of the coefficient matrix = " << ncomp << std::endl;
            }
        }
        if (estimate_ram) {
            double gb;
            if (fmm) {
                // an SL-/ML-FMM project: the reference's cluster set-up and
                // FMM matrix counts for this step (nc_fmm_plan.cpp)
                if (fmm->declare(step, istart, f)) {
                    // the method lines of NC_FrequencyInformations (NC_Main.cpp:1051-1080)
                    const char *name = fmm->method() == 0   ? "Traditional BEM"
                                       : fmm->method() == 1 ? "Single level fast multipole BEM"
                                                            : "Direct multilevel fast multipole BEM";
                    for (std::ostream *o : {(std::ostream *)&std::cout, (std::ostream *)&out}) {
                        *o << "\n" << name << std::endl;
                        if (step == istart) {
                            *o << "\nNumber of equations = " << N << std::endl;
                            if (fmm->method() == 0)
                                *o << "Number of entries of the coefficient matrix = " << (int)((unsigned)N * (unsigned)N)
                                   << std::endl;
                        }
                    }
                }
                fmm->expansion(2.0 * nc::kPI * f / p.c);
                gb = fmm->ram_estimate_gb(std::cout);
            } else {
                // NC_Main.cpp:524-541,717-733: TBEM count, unsigned 32-bit like the reference
                unsigned nint = 0, ncmplx = (unsigned)N;
                std::cout << "TBEM: \n";
                std::cout << "Number of entries right hand side: " << ncmplx << "\n";
                std::cout << "Number of Matrix entries: " << ncmplx * ncmplx << "\n";
                ncmplx += (unsigned)N * (unsigned)N;
                std::cout << "Total Nr. of Integers: " << nint << "\n";
                std::cout << "Total Nr. of Cmplxdble: " << ncmplx << "\n";
                gb = (double)(nint * sizeof(int) + ncmplx * 16) / 1000.0 / 1000.0 / 1000.0;
                std::cout << "RAM Estimation: " << gb << " GByte\n";
            }
            est << step + 1 << " " << f << " " << gb << "\n";
            // device: solver + mesh + evaluation points + a CUDA context
            const double dev = bem_footprint_bytes(N, prec, 0) + bem_mesh_footprint_bytes(N, p.n_sym) +
                               88.0 * (double)ev_nodes.size() + kContextBytes;
            est_gpu << step + 1 << " " << f << " " << dev / 1e9 << "\n";
            continue;
        }
        nc::FreqState fs;
        nc::update_freq(p, f, fs);
        std::vector<cd> bcv(4 * (size_t)N), adm(N);
        for (int d = 0; d < N; ++d) {
            for (int a = 0; a < 4; ++a) bcv[4 * (size_t)d + a] = fs.zbval0[4 * (size_t)be[d] + a];
            adm[d] = fs.zbval1[be[d]];
        }
        bem_frequency_desc fd{};
        fd.wave_number = fs.k;
        fd.time_factor = p.htf;
        fd.tao = p.tao;
        fd.bc_type = bct.data();
        fd.bc_value = reinterpret_cast<const double *>(bcv.data());
        fd.admittance = reinterpret_cast<const double *>(adm.data());
        const int npt = p.n_point > 0 ? p.n_point : 0;
        fd.n_point = npt;
        fd.point_xyz = p.point_xyz.data();
        fd.point_amp = reinterpret_cast<const double *>(fs.zposoc.data());
        fd.n_plane = p.n_plane;
        fd.plane_dir = p.plane_dir.data();
        fd.plane_amp = reinterpret_cast<const double *>(fs.zinwav.data());

        bem_status st = bem_assemble(gpu.solver, &fd);
        if (st != BEM_OK) gpu_fail(out, "assembly", st);
        time(&ltim[4]);
        const time_t lti_est = ltim[4] - ltim[3];
        lti_eqa += lti_est;

        bem_solve_info info{};
        bem_solver_params lim{};
        // NumCalc's default limit is 250 CGS iterations (NC_Main.cpp:83), i.e.
        // 500 matrix-vector products; GMRES spends one product per iteration
        lim.max_iter = nitermax_given ? nitermax : 500;
        bool limited = false;
        if (p.solver == 4) {
            // ISOLVER 4: the direct solver alone, no CGS line (NC_Main.cpp:833-866)
            st = bem_solve_direct(gpu.solver, &info);
            if (st != BEM_OK) gpu_fail(out, "direct solve", st);
        } else if (nitermax_given && nitermax <= 0) {
            limited = true;
            info.iterations = 0;
            info.rel_residual = 1.0;
        } else {
            bem_solver_set_params(gpu.solver, &lim);
            st = bem_solve(gpu.solver, &info);
            if (st == BEM_ERR_NOT_CONVERGED) limited = true;
            else if (st != BEM_OK) gpu_fail(out, "solve", st);
        }
        if (limited) {
            std::cout << "Warning: Maximum number of iterations is reached!\n" << std::endl;
            out << "Warning: Maximum number of iterations is reached!\n" << std::endl;
        }
        if (p.solver != 4)
            out << "\nCGS solver: number of iterations = " << info.iterations << ", relative error = "
                << info.rel_residual << std::endl;
        if (limited) {
            // as NumCalc after a failed CGS (NC_CommonFunctions.cpp:1181-1191)
            std::cout << "Iteration method CGS failed, direct method is used!\n" << std::endl;
            out << "Iteration method CGS failed, direct method is used!\n" << std::endl;
            st = bem_solve_direct(gpu.solver, &info);
            if (st != BEM_OK) gpu_fail(out, "direct solve", st);
        }
        st = bem_get_solution(gpu.solver, reinterpret_cast<double *>(x.data()));
        if (st != BEM_OK) gpu_fail(out, "solution", st);
        time(&ltim[5]);
        const time_t lti_sst = ltim[5] - ltim[4];
        lti_sol += lti_sst;

        // post processing
        char dir[64];
        std::snprintf(dir, sizeof(dir), "be.out/be.%d", step + 1);
        mkdir(dir, kDirMode);
        write_boundary(p, fs, x, dir);
        if (!ev_nodes.empty()) {
            st = bem_project(gpu.solver, (int)ev_nodes.size(), ev_xyz.data(), reinterpret_cast<double *>(pot.data()),
                             reinterpret_cast<double *>(grad.data()));
            if (st != BEM_OK) gpu_fail(out, "projection", st);
            write_eval(p, fs, ev_nodes, pot, grad, dir);
        }
        time(&ltim[6]);
        const time_t lti_pst = ltim[6] - ltim[5];
        lti_pos += lti_pst;
        for (std::ostream *o : {(std::ostream *)&out, (std::ostream *)&std::cout}) {
            if (o == &out) *o << "\nTime Statistic For The Current Step (In Second)\n" << std::endl;
            *o << "Assembling the equation system         : " << lti_est << std::endl;
            *o << "Solving the equation system            : " << lti_sst << std::endl;
            *o << "Post processing                        : " << lti_pst << std::endl;
            *o << "Total                                  : " << lti_est + lti_sst + lti_pst << std::endl;
        }
        std::cout << std::endl;
    }
    if (!estimate_ram) {
        time(&ltim[6]);
        out << "\n\n\n>> T I M E   S T A T I S T I C   (In   Second) <<\n" << std::endl;
        out << "Input                                  : " << ltim[1] - ltim[0] << std::endl;
        out << "Address computation                    : " << ltim[2] - ltim[1] << std::endl;
        out << "Assembling the equation system         : " << lti_eqa << std::endl;
        out << "Solving the equation system            : " << lti_sol << std::endl;
        out << "Post processing                        : " << lti_pos << std::endl;
        out << "The whole job                          : " << ltim[6] - ltim[0] << std::endl;
        std::cout << "\nTime Statistic for the job (in second):" << std::endl;
        std::cout << "Input ............................ " << ltim[1] - ltim[0] << std::endl;
        std::cout << "Address computation .............. " << ltim[2] - ltim[1] << std::endl;
        std::cout << "Assembling the equation system ... " << lti_eqa << std::endl;
        std::cout << "Solving the equation system ...... " << lti_sol << std::endl;
        std::cout << "Post processing .................. " << lti_pos << std::endl;
        std::cout << "The whole job .................... " << ltim[6] - ltim[0] << std::endl;
    }
    return 0;
}

}  // namespace

int main(int argc, char **argv) {
    int istart = 0, iend = 0, nitermax = 250;
    bool estimate_ram = false, check_normals = false, nitermax_given = false;
    for (int i = 1; i < argc; ++i) {
        if (!std::strcmp(argv[i], "-h")) {
            std::printf("-istart   int : start index of iteration\n");
            std::printf("-iend     int : end index of iteration\n");
            std::printf("-nitermax int : max number of CGS iterations\n");
            std::printf("-estimate_ram : estimation the RAM consumption of ML-FMM-BEM and write estimate to "
                        "Memory.txt. Estimate is obtained from the number of non-zeros in the FMM matrices.\n");
            std::printf("-check_normals : check if all normals point to the same domain\n");
            std::printf("-h            : this message\n");
            return 0;
        } else if (!std::strcmp(argv[i], "-istart")) {
            if (++i < argc) istart = std::atoi(argv[i]);
        } else if (!std::strcmp(argv[i], "-iend")) {
            if (++i < argc) iend = std::atoi(argv[i]);
        } else if (!std::strcmp(argv[i], "-nitermax")) {
            if (++i < argc) { nitermax = std::atoi(argv[i]); nitermax_given = true; }
        } else if (!std::strcmp(argv[i], "-estimate_ram")) {
            estimate_ram = true;
        } else if (!std::strcmp(argv[i], "-check_normals")) {
            check_normals = true;
        } else {
            std::cerr << "\nNumCalc was called with an unknown parameter or flag. Use NumCalc -h for help.\n";
            return 255;
        }
    }
    if (istart < 0) {
        std::cerr << "I need to start with a step bigger 0\n";
        return 255;
    }
    std::fprintf(stdout, "istart= %d iend = %d\n", istart, iend);
    time_t lot = time(nullptr);
    tm *d_t = localtime(&lot);
    std::cout << "\n---------- NumCalc (GB300) started: " << d_t->tm_mday << "/" << d_t->tm_mon + 1 << "/"
              << d_t->tm_year + 1900 << " " << d_t->tm_hour << ":" << d_t->tm_min << ":" << d_t->tm_sec
              << " ----------\n" << std::endl;
    char host[150];
    std::memset(host, 0, sizeof(host));
    gethostname(host, sizeof(host) - 1);
    std::cout << "Running on:         " << host << "\n" << std::endl;
    char fname[200];
    if (istart > 0) {
        if (iend >= istart) std::snprintf(fname, sizeof(fname), "NC%d-%d.out", istart, iend);
        else if (iend > 0) {
            std::cerr << "istart is bigger than iend. Stopping now!\n";
            return 255;
        } else std::snprintf(fname, sizeof(fname), "NCfrom%d.out", istart);
    } else {
        if (iend > 0) std::snprintf(fname, sizeof(fname), "NCuntil%d.out", iend);
        else std::snprintf(fname, sizeof(fname), "NC.out");
    }
    std::ofstream out(fname);
    if (!out) {
        std::cout << "can not open the output stream NCout!" << std::endl;
        return 1;
    }
    stamp(out, "\nStart time: ", d_t);
    out << std::endl;
    if (istart == 0 && iend == 0 && !estimate_ram) {
        if (std::system("rm -f -r be.out") == -1) std::cout << "\nCannot create directory be.out";
    }
    mkdir("be.out", kDirMode);
    int rc = 0;
    try {
        rc = run(istart, iend, estimate_ram, check_normals, nitermax, nitermax_given, out);
    } catch (const nc::NcExit &e) {
        if (!e.msg.empty()) {
            std::cout << e.msg << std::endl;
            out << e.msg << std::endl;
        }
        out.close();
        return e.code & 0xff;
    }
    lot = time(nullptr);
    d_t = localtime(&lot);
    stamp(out, "\nEnd time: ", d_t);
    out << std::endl;
    std::cout << "\n---------- NumCalc (GB300) ended: " << d_t->tm_mday << "/" << d_t->tm_mon + 1 << "/"
              << d_t->tm_year + 1900 << " " << d_t->tm_hour << ":" << d_t->tm_min << ":" << d_t->tm_sec
              << " ----------" << std::endl;
    return rc;
}
