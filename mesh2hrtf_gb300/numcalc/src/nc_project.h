// nc_project.h - the drop-in NumCalc's view of a Mesh2HRTF project: the
// NC.inp dialect, the Nodes/Elements files and the derived tables, read with
// the reference NumCalc's rules (mesh2hrtf/NumCalc/src/NC_Input.cpp) so that
// every parsed number, index and table is identical to the reference's.
#pragma once

#include <complex>
#include <fstream>
#include <string>
#include <vector>

namespace nc {

using cd = std::complex<double>;

constexpr int kLineSize = 300;  // fgets buffer, NC_ConstantsVariables.h:46
constexpr int kMaxTerms = 30;   // tokens per line, NC_ConstantsVariables.h:47
constexpr double kPI = 3.1415926535897932385;

// Fatal input error: message for stdout/NC.out and the process exit code
// the reference uses for the same condition.
struct NcExit {
    std::string msg;
    int code;
};

// Line tokenizer with NC_GetLine semantics (NC_Input.cpp:1596-1631): split on
// ' ' only, drop the line's last character (the newline), a '#' anywhere in
// the first token makes the line a comment, tokens persist between calls.
class LineReader {
public:
    explicit LineReader(FILE *f) : f_(f) {}
    int next();                       // number of tokens (0: empty/comment)
    int next_nonempty();              // while(!NC_GetLine(...))
    const std::string &operator[](int i) const { return terms_[i]; }

private:
    FILE *f_;
    std::string terms_[kMaxTerms];
};

int to_int(const std::string &s);     // NC_String2Integer, NC_Input.cpp:1635-1655
double to_double(const std::string &s);  // NC_String2Double, NC_Input.cpp:1659-1683

struct BcLine {
    int low, high;
    std::string keyword;
    double re, im;
    bool ref;
    int re_curve, im_curve;
};

struct Project {
    // header
    std::string version, title;
    int n_freq = 0;
    double step_increment = 0.0, first_step = 0.0;
    std::vector<double> freqs;
    // main parameters
    int n_groups = 0, n_elem = 0, n_nodes = 0, min_fmm_terms = 0, n_sym = 0, method_bem = 0, solver = 0;
    int n_plane = 0, n_point = 0, interior = 0, precond = 0, scan_degree = 0;
    double clus_edge = 0.0, c = 0.0, rho = 0.0, htf = 1.0, tao = 1.0;
    int n_reflections = 1;
    // mesh (internal order = file order)
    std::vector<int> node_ext;
    std::vector<double> node_xyz;        // [n_nodes][3]
    std::vector<int> node_class;         // >= 0 BE node index, -1 evaluation node
    std::vector<int> elem_ext, elem_nv, elem_prop, elem_group;
    std::vector<int> elem_conn;          // [n_elem][4], internal node indices
    std::vector<double> centel, elenor, areael;  // [n][3], [n][15], [n]
    int n_be = 0, n_ev = 0, n_nodes_be = 0, n_nodes_ev = 0;
    double avg_area = 0.0, diameter = 0.0;
    int sym_planes[3] = {0, 0, 0};
    double sym_coords[3] = {0, 0, 0};
    std::vector<int> group_index, group_count, group_prop;
    // boundary conditions (NC_StoreBoundaryConditions)
    std::vector<int> ibval;
    std::vector<cd> zbvao0;              // [n_elem][4]
    std::vector<cd> zbvao1, zbvao2;
    std::vector<int> ibvcurv;            // [n_elem][6]
    // sources
    std::vector<int> plane_id, point_id;
    std::vector<double> plane_dir, point_xyz;
    std::vector<cd> plane_amp0, point_amp0;
    std::vector<int> plane_curve, point_curve;  // [n][2]
    // curves
    std::vector<int> curve_id, curve_npts;
    std::vector<std::vector<double>> curve_f, curve_fac;
    // diagnostics written by NC_WriteParameters
    double freq_max = 0.0, dmesh_max = 0.0, dmesh_min = 0.0, dmesh_ave = 0.0;
};

// Reads NC.inp (already opened) and the mesh files it lists, in the
// reference's order; writes the parameter echo to NCout.  Throws NcExit.
void read_project(FILE *inp, std::ofstream &ncout, bool check_normals, Project &p);

// Per-frequency boundary data after NC_UpdateFreqCurves
// (NC_EquationSystem.cpp:1815-1961).
struct FreqState {
    double frequency, omega, k, rpfact;
    std::vector<cd> zbval0, zbval1;      // [n_elem][4], [n_elem]
    std::vector<cd> zinwav, zposoc;
};
void update_freq(const Project &p, double frequency, FreqState &s);

// Writes the parsed tables (records: name[24], dtype[8], int64 count, data)
// for parser parity checks.
void dump_tables(const Project &p, const char *path);

}  // namespace nc
