// nc_project.cpp - NC.inp / Nodes.txt / Elements.txt reader of the drop-in
// NumCalc.  Every rule below restates the reference's input routines
// (mesh2hrtf/NumCalc/src/NC_Input.cpp, cited per function) so that the
// parsed project is identical, including its quirks: tokens split on ' '
// only, the last character of every line dropped, tokens persisting from the
// previous line, atoi/atof conversions, first-match node numbering.
// Compiled with -ffp-contract=off: the geometry below rounds like the
// reference's x86 build.
#include "nc_project.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <unordered_map>

namespace nc {

namespace {

[[noreturn]] void die(const std::string &msg, int code = 1) { throw NcExit{msg, code}; }

std::string fmt_i(const std::string &a, int v) { return a + std::to_string(v); }

std::string fmt_d(const std::string &a, double v) {
    std::ostringstream o;
    o << a << v;
    return o.str();
}

[[noreturn]] void die1(const std::string &msg, const std::string &s1, int v1) {
    die(msg + "\n" + fmt_i(s1, v1));
}

[[noreturn]] void die2(const std::string &msg, const std::string &s1, int v1, const std::string &s2, int v2) {
    die(msg + "\n" + fmt_i(s1, v1) + "\n" + fmt_i(s2, v2));
}

void warn(std::ofstream &out, const std::string &msg, const std::string &body) {
    std::cout << "\nWarning: " << msg << std::endl << body << "\n" << std::endl;
    out << "\nWarning: " << msg << std::endl << body << "\n" << std::endl;
}

// NC_ComputeGlobalCoordinates / NC_ComputeUnitVectorOnElement,
// NC_3dFunctions.cpp:95-178.
void shape(int nv, double s, double t, double *sh, double *ds, double *dt) {
    if (nv == 3) {
        sh[0] = s; sh[1] = t; sh[2] = 1.0 - s - t;
        ds[0] = dt[1] = 1.0; ds[1] = dt[0] = 0.0; ds[2] = dt[2] = -1.0;
    } else {
        double s1 = 0.25 * (s + 1.0), s2 = 0.25 * (s - 1.0), t1 = t + 1.0, t2 = t - 1.0;
        sh[0] = s1 * t1; sh[1] = -s2 * t1; sh[2] = s2 * t2; sh[3] = -s1 * t2;
        ds[0] = 0.25 * (t + 1.0); ds[2] = 0.25 * (t - 1.0); ds[1] = -ds[0]; ds[3] = -ds[2];
        dt[0] = 0.25 * (s + 1.0); dt[2] = 0.25 * (s - 1.0); dt[1] = -dt[2]; dt[3] = -dt[0];
    }
}

double normal_at(int nv, const double p[4][3], double s, double t, double *nrm) {
    double sh[4], ds[4], dt[4], a[3], b[3];
    shape(nv, s, t, sh, ds, dt);
    for (int i = 0; i < 3; ++i) {
        a[i] = b[i] = 0.0;
        for (int j = 0; j < nv; ++j) { a[i] += ds[j] * p[j][i]; b[i] += dt[j] * p[j][i]; }
    }
    nrm[0] = a[1] * b[2] - b[1] * a[2];
    nrm[1] = a[2] * b[0] - b[2] * a[0];
    nrm[2] = a[0] * b[1] - b[0] * a[1];
    double len = std::sqrt(nrm[0] * nrm[0] + nrm[1] * nrm[1] + nrm[2] * nrm[2]);
    nrm[0] /= len; nrm[1] /= len; nrm[2] /= len;
    return len;
}

const double CSI8[8] = {1.0, -1.0, -1.0, 1.0, 0.0, -1.0, 0.0, 1.0};
const double ETA8[8] = {1.0, 1.0, -1.0, -1.0, 1.0, 0.0, -1.0, 0.0};
const double CSI6[6] = {1.0, 0.0, 0.0, 0.5, 0.0, 0.5};
const double ETA6[6] = {0.0, 1.0, 0.0, 0.5, 0.5, 0.0};

// NC_ComputeFrequencies, NC_Input.cpp:1686-1732.
void compute_frequencies(Project &p, const std::vector<double> &ctime, const std::vector<double> &cfreq) {
    const int np = (int)ctime.size();
    p.freqs.assign(p.n_freq, 0.0);
    for (int i = 0; i < p.n_freq; ++i) {
        double t = p.first_step + (double)(i + 1) * p.step_increment;
        if (ctime[0] >= t) { p.freqs[i] = cfreq[0]; continue; }
        int j1 = -1;
        for (int j = 1; j < np; ++j) {
            if (ctime[j] > t) { j1 = j; break; }
            else if (ctime[j] == t) { p.freqs[i] = cfreq[j]; j1 = np; break; }
        }
        if (j1 == -1) p.freqs[i] = cfreq[np - 1];
        else if (j1 < np)
            p.freqs[i] = cfreq[j1 - 1] + (t - ctime[j1 - 1]) * (cfreq[j1] - cfreq[j1 - 1]) / (ctime[j1] - ctime[j1 - 1]);
    }
}

}  // namespace

int LineReader::next() {
    char buf[kLineSize];
    if (std::fgets(buf, kLineSize, f_) == nullptr) die("\nError parsing the input file", -1);
    std::string line(buf);
    int nn = 0, ss = 0, ii = 0;
    const int len = (int)line.length() - 1;
    while (nn < len) {
        nn = (int)line.find(' ', ss);
        if (nn == -1) nn = len;
        if (nn - ss > 0 && ii < kMaxTerms) terms_[ii++] = line.substr(ss, nn - ss);
        ss = nn + 1;
    }
    if ((int)terms_[0].find("#", 0) >= 0) ii = 0;
    return ii;
}

int LineReader::next_nonempty() {
    int n;
    while (!(n = next())) {
    }
    return n;
}

int to_int(const std::string &s) {
    if ((int)s.length() > 15) die("Length of the string > n_chwk!\nThe string: " + s);
    return std::atoi(s.c_str());
}

double to_double(const std::string &s) {
    if ((int)s.length() > 25) die("Length of the string > n_chwk!\nThe string: " + s);
    return std::atof(s.c_str());
}

// NC_ReadBasicParametersA/B (NC_Input.cpp:151-347), NC_ReadMesh (353-737),
// NC_checkedges (741-789), NC_ReadBoundaryConditions (792-880),
// NC_ReadSoundSources (1002-1070), NC_ReadFrequencyCurves (1073-1160),
// NC_StoreBoundaryConditions (1163-1406), NC_WriteParameters (1409-1593).
void read_project(FILE *inp, std::ofstream &out, bool check_normals, Project &p) {
    LineReader L(inp);
    // ---- version and title
    int nt = L.next_nonempty();
    if (L[0] != "Mesh2HRTF") die("Key word Mesh2HRTF expected!");
    p.version = L[0];
    for (int i = 1; i < nt; ++i) p.version += " " + L[i];
    nt = L.next_nonempty();
    p.title = L[0];
    for (int i = 1; i < nt; ++i) p.title += " " + L[i];
    std::cout << "Job title: " << p.title << std::endl;
    L.next_nonempty();  // control parameter I
    L.next_nonempty();  // control parameter II
    p.n_freq = to_int(L[1]);
    p.step_increment = to_double(L[2]);
    p.first_step = to_double(L[3]);
    // ---- frequency curve
    L.next_nonempty();
    const int npc = to_int(L[1]);
    std::vector<double> ctime(npc > 0 ? npc : 0), cfreq(npc > 0 ? npc : 0);
    for (int i = 0; i < npc; ++i) {
        L.next_nonempty();
        ctime[i] = to_double(L[0]);
        cfreq[i] = to_double(L[1]);
    }
    if (npc <= 0 && p.n_freq > 0) die("frequency curve without points");
    compute_frequencies(p, ctime, cfreq);
    // ---- main parameters I
    L.next_nonempty();
    p.n_groups = to_int(L[0]);
    p.n_elem = to_int(L[1]);
    p.n_nodes = to_int(L[2]);
    p.min_fmm_terms = to_int(L[3]);
    p.n_sym = to_int(L[4]);
    p.method_bem = to_int(L[7]);
    p.solver = to_int(L[8]);
    if (p.n_elem < 1) die1("Number of elements must > 0!", "Number of elements = ", p.n_elem);
    if (p.n_nodes < 1) die1("Number of nodes must > 0!", "Number of nodes = ", p.n_nodes);
    if (p.min_fmm_terms == 0) p.min_fmm_terms = 8;
    if (p.min_fmm_terms < 5 || p.min_fmm_terms > 10)
        die1("minExpansionTermsFMM_  must be in [5 10]!", "minExpansionTermsFMM_ = ", p.min_fmm_terms);
    if (p.n_sym < 0 || p.n_sym > 3)
        die1("Number of symmetry planes must be in [0 3]!", "Number of symmetry planes = ", p.n_sym);
    if (p.solver < 0 || p.solver > 4) die1("ISOLVER must be 0 or 4!", "ISOLVER = ", p.solver);
    if (p.solver > 0 && p.solver < 4) die1("ISOLVER must be 0 or 4!", "ISOLVER = ", p.solver);
    if (p.method_bem != 0 && p.method_bem != 1 && p.method_bem != 4)
        die1("methodBEM_ must be in {0,1,4}!", "methodBEM_ = ", p.method_bem);
    if (p.method_bem != 0 && p.solver == 4) p.solver = 0;
    // ---- main parameters II
    L.next_nonempty();
    p.n_plane = to_int(L[0]);
    p.n_point = to_int(L[1]);
    p.interior = to_int(L[2]);
    p.clus_edge = to_double(L[3]);
    p.precond = to_int(L[4]);
    if (p.n_plane < 0)
        die1("Number of the incident plane waves must >= 0!", "Number of the incident plane waves = ", p.n_plane);
    if (p.n_point < -1)
        die1("Number of the point sources must >= -1!", "Number of the point sources = ", p.n_plane);
    if (p.interior != 0 && p.interior != 1) die1("IFINTE must = 0 or 1!", "IFINTE = ", p.interior);
    if (p.precond < -3 || p.precond > 2) die1("IPRECOND must be in [-3 2]!", "IPRECOND = ", p.precond);
    if (p.precond <= -3) { p.scan_degree = 3; p.precond = 0; }
    else if (p.precond == -2) { p.scan_degree = 2; p.precond = 0; }
    else if (p.precond == -1) { p.scan_degree = 1; p.precond = 0; }
    else p.scan_degree = 0;
    if (p.solver == 4) p.precond = 2;
    L.next_nonempty();  // main parameters III
    L.next_nonempty();  // main parameters IV
    p.c = to_double(L[0]);
    p.rho = to_double(L[1]);
    p.htf = to_double(L[2]);
    if (p.htf != -1.0) p.htf = 1.0;
    if (p.c < 300.0) warn(out, "speedOfSound_ perhaps too small!", fmt_d("speedOfSound_ = ", p.c));
    if (p.rho < 1.0) warn(out, "densityOfMedium_ perhaps too small!", fmt_d("densityOfMedium_ = ", p.rho));
    p.n_reflections = (int)std::pow(2.0, p.n_sym);
    p.tao = p.interior ? -1.0 : 1.0;

    // ---- NODES
    const int NN = p.n_nodes, NE = p.n_elem;
    p.node_ext.assign(NN, 0);
    p.node_xyz.assign(3 * (size_t)NN, 0.0);
    L.next_nonempty();
    if (L[0] != "NODES") die("Key word NODES expected!");
    int i = 0;
    while (i < NN) {
        L.next_nonempty();
        FILE *tf = std::fopen(L[0].c_str(), "r");
        if (!tf) die("No Nodes file found!", -1);
        LineReader T(tf);
        T.next_nonempty();
        const int cnt = to_int(T[0]);
        for (int jj = 0; jj < cnt; ++jj) {
            T.next_nonempty();
            if (i >= NN) { std::fclose(tf); die("more nodes in the files than in Main Parameters I"); }
            p.node_ext[i] = to_int(T[0]);
            p.node_xyz[3 * (size_t)i] = to_double(T[1]);
            p.node_xyz[3 * (size_t)i + 1] = to_double(T[2]);
            p.node_xyz[3 * (size_t)i + 2] = to_double(T[3]);
            ++i;
        }
        std::fclose(tf);
    }
    // ---- ELEMENTS
    p.elem_ext.assign(NE, 0);
    p.elem_nv.assign(NE, 0);
    p.elem_prop.assign(NE, 0);
    p.elem_group.assign(NE, 0);
    p.elem_conn.assign(4 * (size_t)NE, -1);
    L.next_nonempty();
    if (L[0] != "ELEMENTS") die("Key word ELEMENTS expected!");
    i = 0;
    while (i < NE) {
        L.next_nonempty();
        FILE *tf = std::fopen(L[0].c_str(), "r");
        if (!tf) die("No Elements file found!", -1);
        LineReader T(tf);
        T.next_nonempty();
        const int cnt = to_int(T[0]);
        for (int jj = 0; jj < cnt; ++jj) {
            const int n = T.next_nonempty();
            if (n < 7 || n > 8) {
                std::fclose(tf);
                die2("number of entris of a input line must be 7 or 8!",
                     "number of the element under the key word ELEMENTS = ", to_int(T[0]),
                     "number of entrie of the line = ", n);
            }
            if (i >= NE) { std::fclose(tf); die("more elements in the files than in Main Parameters I"); }
            p.elem_ext[i] = to_int(T[0]);
            p.elem_nv[i] = n - 4;
            for (int j = 0; j < p.elem_nv[i]; ++j) p.elem_conn[4 * (size_t)i + j] = to_int(T[j + 1]);
            p.elem_prop[i] = to_int(T[n - 3]);
            p.elem_group[i] = to_int(T[n - 1]);
            ++i;
        }
        std::fclose(tf);
    }
    // ---- BE / evaluation elements
    p.n_be = p.n_ev = 0;
    {
        int g0 = 0, k0 = 0;
        for (i = 0; i < NE; ++i) {
            if (p.elem_prop[i] == 0) ++p.n_be;
            else if (p.elem_prop[i] == 2) {
                if (p.n_ev == 0) { g0 = p.elem_group[i]; k0 = i; }
                else if (p.elem_group[i] != g0) {
                    std::ostringstream m;
                    m << "\nElement " << p.elem_ext[k0] << " belongs to the el. group " << p.elem_group[k0]
                      << " but\nElement " << p.elem_ext[i] << " belongs to the el. group " << p.elem_group[i]
                      << "!\nElements of the evaluation mesh must be of the same el. group!";
                    die(m.str());
                }
                ++p.n_ev;
            } else {
                die2("listElementProperty[i] must be 0 or 2!", "i = ", i, "listElementProperty[i] = ", p.elem_prop[i]);
            }
        }
    }
    // ---- symmetry planes
    if (p.n_sym > 0) {
        L.next_nonempty();
        if (L[0] != "SYMMETRY") die("Key word SYMMETRY expected!");
        L.next_nonempty();
        for (int k = 0; k < 3; ++k) p.sym_planes[k] = to_int(L[k]);
        L.next_nonempty();
        for (int k = 0; k < 3; ++k) p.sym_coords[k] = to_double(L[k]);
        int cnt = 0;
        for (int k = 0; k < 3; ++k) {
            if (p.sym_planes[k]) ++cnt;
            switch (p.sym_planes[k]) {
            case 0: case 1: break;
            case 2: p.sym_planes[k] = -1; break;
            case 3: p.sym_planes[k] = 2; break;
            case 4: p.sym_planes[k] = -2; break;
            default:
                die2("listSymmetryPlanes[i] must be equal to 0, 1, 2, 3, or 4!", "i = ", k,
                     "listSymmetryPlanes[i] = ", p.sym_planes[k]);
            }
        }
        if (cnt != p.n_sym) die2("j must equal to numSymmetricPlanes_", "j = ", cnt, "numSymmetricPlanes_ = ", p.n_sym);
    }
    // ---- external -> internal node numbers, first match in file order
    {
        std::unordered_map<int, int> first;
        first.reserve(2 * (size_t)NN);
        for (int k = NN - 1; k >= 0; --k) first[p.node_ext[k]] = k;
        for (i = 0; i < NE; ++i)
            for (int j = 0; j < p.elem_nv[i]; ++j) {
                auto it = first.find(p.elem_conn[4 * (size_t)i + j]);
                if (it == first.end())
                    die2("Node of element does not exist in the connectivity list!", "Number of element = ",
                         p.elem_ext[i], "Local number of the node in the element = ", j);
                p.elem_conn[4 * (size_t)i + j] = it->second;
            }
    }
    if (check_normals) {
        std::vector<int> hedges(NN, 0);
        bool ok = true;
        for (int e = 0; e < NE; ++e) {
            if (p.elem_prop[e] == 2) continue;
            const int nv = p.elem_nv[e];
            const int *c = &p.elem_conn[4 * (size_t)e];
            for (int j = 0; j < nv - 1; ++j) { hedges[c[j]] -= c[j + 1] + 1; hedges[c[j + 1]] += c[j] + 1; }
            hedges[c[nv - 1]] -= c[0] + 1;
            hedges[c[0]] += c[nv - 1] + 1;
        }
        for (int j = 0; j < NN; ++j)
            if (hedges[j] != 0) {
                std::cerr << "Problem with element containing the node " << p.node_ext[j] << "\n";
                ok = false;
            }
        if (!ok) die("There seems to be at least one element that is differently ordered to the rest");
    }
    // ---- centres, normals, areas
    p.centel.assign(3 * (size_t)NE, 0.0);
    p.elenor.assign(15 * (size_t)NE, 0.0);
    p.areael.assign(NE, 0.0);
    double area_ev = 0.0;
    int nbouel = 0, nevlel = 0;
    p.avg_area = 0.0;
    for (i = 0; i < NE; ++i) {
        const int pr = p.elem_prop[i];
        if (pr < 0 || pr > 2 || pr == 1)
            die2("listElementProperty[i] must be equal to 0 or 2!", "number of the element = ", p.elem_ext[i],
                 "listElementProperty[i] = ", pr);
        const int nv = p.elem_nv[i];
        double pts[4][3] = {{0}};
        for (int j = 0; j < nv; ++j)
            for (int k = 0; k < 3; ++k) pts[j][k] = p.node_xyz[3 * (size_t)p.elem_conn[4 * (size_t)i + j] + k];
        double s, t, are0;
        if (nv == 3) { s = t = 1.0 / 3.0; are0 = 0.5; }
        else if (nv == 4) { s = t = 0.0; are0 = 4.0; }
        else die2("Number of nodes of an element must be 3 or 4!", "number of nodes of the element = ", nv,
                  "number of the element = ", p.elem_ext[i]);
        double sh[4], ds[4], dt[4], nrm[3];
        shape(nv, s, t, sh, ds, dt);
        for (int k = 0; k < 3; ++k) {
            double acc = 0.0;
            for (int j = 0; j < nv; ++j) acc += sh[j] * pts[j][k];
            p.centel[3 * (size_t)i + k] = acc;
        }
        const double leng = normal_at(nv, pts, s, t, nrm);
        for (int k = 0; k < 3; ++k) p.elenor[15 * (size_t)i + k] = nrm[k];
        p.areael[i] = leng * are0;
        if (pr == 2) { area_ev += p.areael[i]; ++nevlel; }
        else { p.avg_area += p.areael[i]; ++nbouel; }
        for (int j = 0; j < nv; ++j) {
            const double sj = nv == 3 ? CSI6[j] : CSI8[j], tj = nv == 3 ? ETA6[j] : ETA8[j];
            normal_at(nv, pts, sj, tj, nrm);
            for (int k = 0; k < 3; ++k) p.elenor[15 * (size_t)i + 3 * (j + 1) + k] = nrm[k];
        }
    }
    p.avg_area /= (double)nbouel;
    // ---- node classes
    p.node_class.assign(NN, -3);
    for (i = 0; i < NE; ++i)
        if (p.elem_prop[i] == 0)
            for (int j = 0; j < p.elem_nv[i]; ++j) p.node_class[p.elem_conn[4 * (size_t)i + j]] = 1;
    for (i = 0; i < NE; ++i)
        if (p.elem_prop[i] == 2)
            for (int j = 0; j < p.elem_nv[i]; ++j) {
                int &c = p.node_class[p.elem_conn[4 * (size_t)i + j]];
                if (c != 1) c = -1;
                else die1("BE mesh and evaluation mesh have common node!", "Number of the common node = ",
                          p.node_ext[p.elem_conn[4 * (size_t)i + j]]);
            }
    p.n_nodes_be = p.n_nodes_ev = 0;
    for (i = 0; i < NN; ++i) {
        if (p.node_class[i] == 1) p.node_class[i] = p.n_nodes_be++;
        else if (p.node_class[i] == -1) ++p.n_nodes_ev;
        else if (p.node_class[i] == -3) {
            std::ostringstream m;
            m << "\nnumber of the isolated node: " << p.node_ext[i] << "\nIsolated node found!";
            die(m.str());
        }
    }
    if (p.n_nodes_be == 0) die("Number of boundary elements is zero!");
    // ---- diameter of the BE mesh (symmetry-aware)
    {
        double mm[3][2];
        const double dtl = std::sqrt(p.avg_area) / 100.0;
        for (int j = 0; j < 3; ++j) { mm[j][0] = -9.9e20; mm[j][1] = 9.9e20; }
        for (i = 0; i < NN; ++i) {
            if (p.node_class[i] < 0) continue;
            for (int j = 0; j < 3; ++j) {
                const double v = p.node_xyz[3 * (size_t)i + j];
                if (v > mm[j][0]) mm[j][0] = v;
                if (v < mm[j][1]) mm[j][1] = v;
            }
        }
        for (int j = 0; j < 3; ++j) {
            if (p.n_sym == 0 || p.sym_planes[j] == 0) {
                mm[j][0] -= mm[j][1];
            } else if (std::abs(p.sym_planes[j]) <= 2) {
                const double sc = p.sym_coords[j];
                if (mm[j][0] >= sc - dtl && mm[j][1] >= sc - dtl) mm[j][0] = 2.0 * (mm[j][0] - sc);
                else if (mm[j][0] <= sc + dtl && mm[j][1] <= sc + dtl) mm[j][0] = 2.0 * (sc - mm[j][1]);
                else die("All BE nodes must be located on the same side of a symmetric plane!");
            }
        }
        p.diameter = 0.0;
        for (int j = 0; j < 3; ++j) p.diameter += mm[j][0] * mm[j][0];
        p.diameter = std::sqrt(p.diameter);
    }
    // ---- element groups in first-appearance order
    {
        std::vector<int> idx, prop;
        for (i = 0; i < NE; ++i) {
            bool seen = false;
            for (size_t j = 0; j < idx.size(); ++j)
                if (p.elem_group[i] == idx[j]) { seen = true; break; }
            if (!seen) { idx.push_back(p.elem_group[i]); prop.push_back(p.elem_prop[i]); }
        }
        if ((int)idx.size() < p.n_groups) p.n_groups = (int)idx.size();
        else if ((int)idx.size() > p.n_groups)
            die2("ielgrp must be less than or equal to nelgrp", "ielgrp = ", (int)idx.size(), "nelgrp = ", p.n_groups);
        p.group_index.assign(idx.begin(), idx.begin() + p.n_groups);
        p.group_prop.assign(prop.begin(), prop.begin() + p.n_groups);
        p.group_count.assign(p.n_groups, 0);
        for (i = 0; i < NE; ++i)
            for (int j = 0; j < p.n_groups; ++j)
                if (p.elem_group[i] == p.group_index[j]) { ++p.group_count[j]; break; }
    }

    // ---- BOUNDARY ... RETU
    std::vector<BcLine> bcl;
    {
        L.next_nonempty();
        if (L[0] != "BOUNDARY") die("Key word BOUNDARY expected!");
        const int maxl = 2 * p.n_be;
        bool retu = false;
        for (i = 0; i < maxl; ++i) {
            const int n = L.next_nonempty();
            if (L[0] == "RETU") { retu = true; break; }
            if (n < 9) die1("A input line under BOUNDARY is too short!", "Number of the input line = ", i);
            if (L[0] != "ELEM") die("Key word ELEM expected!");
            BcLine b;
            b.low = to_int(L[1]);
            if (L[2] != "TO") die("Key word TO expected!");
            b.high = to_int(L[3]);
            b.keyword = L[4];
            if ((L[6] == "-1" && L[8] != "-1") || (L[6] != "-1" && L[8] == "-1"))
                die("ERROR: Curves have to be specified for all parts of a Boundary or Source. I.e., ALL curve "
                    "numbers in one line must be -1 or ALL curve numbers must not be -1");
            b.re = to_double(L[5]);
            b.ref = false;
            b.re_curve = b.im_curve = 0;
            if (L[6] != "-1") { b.ref = true; b.re_curve = to_int(L[6]); }
            b.im = to_double(L[7]);
            if (L[8] == "-1") b.ref = false;
            else { b.ref = true; b.im_curve = to_int(L[8]); }
            bcl.push_back(b);
        }
        if (!retu) die("Key word RETU expected!");
    }
    // ---- sound sources
    if (p.n_plane > 0 || p.n_point > 0 || p.n_point == -1) {
        if (p.n_plane > 0) {
            L.next_nonempty();
            if (L[0] != "PLANE") die("Key word PLANE WAVE expected!");
            for (i = 0; i < p.n_plane; ++i) {
                const int n = L.next_nonempty();
                if (n != 8)
                    die2("Number of terms of an input line for plane wave must be 8!", "Number of terms = ", n,
                         "Number of the input line under the key word PLANE WAVE = ", i + 1);
                p.plane_id.push_back(to_int(L[0]));
                double d[3] = {to_double(L[1]), to_double(L[2]), to_double(L[3])};
                double len = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                d[0] /= len; d[1] /= len; d[2] /= len;
                for (int k = 0; k < 3; ++k) p.plane_dir.push_back(d[k]);
                p.plane_amp0.push_back(cd(to_double(L[4]), to_double(L[6])));
                p.plane_curve.push_back(to_int(L[5]));
                p.plane_curve.push_back(to_int(L[7]));
            }
        }
        if (p.n_point > 0) {
            L.next_nonempty();
            if (L[0] != "POINT") die("Key word POINT SOURCES expected!");
            for (i = 0; i < p.n_point; ++i) {
                const int n = L.next_nonempty();
                if (n != 8)
                    die2("Number of terms of an input line for pont source must be 8!", "Number of terms = ", n,
                         "Number of the input line under the key word POINT SOURCE = ", i + 1);
                p.point_id.push_back(to_int(L[0]));
                for (int k = 1; k <= 3; ++k) p.point_xyz.push_back(to_double(L[k]));
                p.point_amp0.push_back(cd(to_double(L[4]), to_double(L[6])));
                p.point_curve.push_back(to_int(L[5]));
                p.point_curve.push_back(to_int(L[7]));
            }
        }
    }
    // ---- CURVES / POST PROCESS / END
    p.ibvcurv.assign(6 * (size_t)NE, -1);
    {
        L.next_nonempty();
        bool curves = false;
        if (L[0] == "CURVES") curves = true;
        else if (L[0] != "POST") die("Key word CURVES or POST PROCESS expected!");
        int ncv = 0;
        if (curves) {
            const int n = L.next_nonempty();
            if (n != 2)
                die1("Number of terms of the input line direct under the key word CURVE must be 2!",
                     "Number of terms = ", n);
            ncv = to_int(L[0]);
            if (ncv < 0) ncv = 0;
            for (i = 0; i < ncv; ++i) {
                const int n2 = L.next_nonempty();
                if (n2 != 2)
                    die2("Number of terms of the firs input line for a curve must be 2!", "Number of terms = ", n2,
                         "number of the curve = ", i);
                p.curve_id.push_back(to_int(L[0]));
                const int np = to_int(L[1]);
                p.curve_npts.push_back(np);
                p.curve_f.emplace_back();
                p.curve_fac.emplace_back();
                for (int j = 0; j < np; ++j) {
                    L.next_nonempty();
                    p.curve_f.back().push_back(to_double(L[0]));
                    p.curve_fac.back().push_back(to_double(L[1]));
                }
            }
            L.next_nonempty();
            if (L[0] != "POST") die("Key word POST PROCESS expected!");
        }
        int n = 0;
        while (n == 0 || n > 1 || (n == 1 && L[0] != "END")) n = L.next();
    }
    // ---- store boundary conditions
    {
        int maxnuel = 0;
        for (i = 0; i < NE; ++i) maxnuel = std::max(maxnuel, p.elem_ext[i]);
        if (maxnuel > 10000000) {
            out << "\nWarning: external element number too large!\nThe maximun value = " << maxnuel << std::endl;
            std::cout << "\nWarning: external element number too large!\nThe maximun value = " << maxnuel << std::endl;
        }
        std::unordered_map<int, int> g2l;
        for (i = NE - 1; i >= 0; --i)
            if (p.elem_prop[i] != 2) g2l[p.elem_ext[i]] = i;
        p.ibval.assign(NE, 0);
        p.zbvao0.assign(4 * (size_t)NE, cd(0.0, 0.0));
        p.zbvao1.assign(NE, cd(0.0, 0.0));
        p.zbvao2.assign(NE, cd(0.0, 0.0));
        std::vector<int> impecurve(p.curve_id.size(), 0);
        for (size_t li = 0; li < bcl.size(); ++li) {
            const BcLine &b = bcl[li];
            int nbtyp = 0;
            bool ifimpe = false;
            if (b.keyword == "VELO") nbtyp = 0;
            else if (b.keyword == "PRES") nbtyp = 1;
            else if (b.keyword == "ADMI") nbtyp = 2;
            else if (b.keyword == "IMPE") { nbtyp = 2; ifimpe = true; }
            else if (b.keyword == "TRAD") die("Transfer admittance boundary condition is not supported!");
            else if (b.keyword == "TRIM") die("Transfer impedance boundary condition is not supported!");
            else {
                std::cout << "The false key word = " << b.keyword << std::endl;
                out << "The false key word = " << b.keyword << std::endl;
                die1("False key word in a input line for boundary conditions!", "Input line number = ", (int)li + 1);
            }
            double reap = b.re, imgp = b.im;
            if (ifimpe && reap == 0 && imgp == 0) { ifimpe = false; nbtyp = 1; }
            if (b.ref && ifimpe) {
                std::cerr << "Sorry Impedance boundary conditions in CURVES is not implemented yet. Please use ADMI "
                             "conditions. They work with CURVES. Sorry for the inconvinience.\n";
                throw NcExit{"", -1};
            }
            if (ifimpe) {
                const double dwk = reap * reap + imgp * imgp;
                reap /= dwk;
                imgp /= (-dwk);
            }
            for (int j = b.low; j <= b.high; ++j) {
                auto it = g2l.find(j);
                if (it == g2l.end()) continue;
                const int j1 = it->second;
                switch (nbtyp) {
                case 0:
                    for (int k = 0; k < p.elem_nv[j1]; ++k) p.zbvao0[4 * (size_t)j1 + k] = cd(reap, imgp);
                    break;
                case 1:
                    for (int k = 0; k < p.elem_nv[j1]; ++k) p.zbvao0[4 * (size_t)j1 + k] = cd(reap, imgp);
                    p.ibval[j1] = 1;
                    break;
                case 2:
                    p.zbvao1[j1] = cd(reap, imgp);
                    if (b.ref) {
                        p.ibvcurv[6 * (size_t)j1 + 2] = b.re_curve;
                        p.ibvcurv[6 * (size_t)j1 + 3] = b.im_curve;
                    }
                    if (p.ibval[j1] == 0) p.ibval[j1] = 2;
                    else if (p.ibval[j1] == 1)
                        std::cout << "Warning; for el. " << j << " the pressure boundary condition is "
                                  << "prescribed, the additional admittance boundary condition is ignored!"
                                  << std::endl;
                    else if (p.ibval[j1] == 3) p.ibval[j1] = 4;
                    break;
                }
            }
            if (ifimpe && b.ref) {
                impecurve[b.re_curve] = 1;
                impecurve[b.im_curve] = 1;
            }
        }
        for (size_t c = 0; c < p.curve_id.size(); ++c)
            if (impecurve[c])
                for (int j = 0; j < p.curve_npts[c]; ++j) {
                    double &v = p.curve_fac[c][j];
                    if (std::fabs(v) > 1.0e-10) v = 1.0 / v;
                    else v = v >= 0.0 ? 1.0e10 : -1.0e10;
                }
    }

    // ---- parameter echo (NC_WriteParameters, NC_Input.cpp:1409-1593)
    {
        int k1 = 0;
        double dmax = 0.0, dmin = 1.0e20, dave = 0.0, deqi = 0.0;
        for (i = 0; i < NE; ++i) {
            int j1 = p.elem_nv[i];
            if (j1 != 3 && j1 != 4) die1("An element must have 3 or 4 nodes!", "Number of the false element = ", p.elem_ext[i]);
            if (p.elem_prop[i] == 2) continue;
            if (p.areael[i] < 0.0)
                die2("Element with negative area is found!", "external elemen number = ", p.elem_ext[i],
                     "internal element number = ", i);
            double dref = std::sqrt(p.areael[i]);
            if (j1 == 3) dref *= 1.51967;
            for (int j = 0; j < j1; ++j) {
                int k = j + 1 == j1 ? 0 : j + 1;
                const double *a = &p.node_xyz[3 * (size_t)p.elem_conn[4 * (size_t)i + j]];
                const double *b = &p.node_xyz[3 * (size_t)p.elem_conn[4 * (size_t)i + k]];
                const double dist =
                    std::sqrt((a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]) + (a[2] - b[2]) * (a[2] - b[2]));
                if (dist > dmax) dmax = dist;
                if (dist < dmin) dmin = dist;
                dave += dist;
                deqi += j1 == 3 ? dist * 0.748 : dist;
                if (dist > dref * 10.0 && dist < dref * 100.0)
                    warn(out, "Element with very long side found!",
                         fmt_i("external elemen number = ", p.elem_ext[i]) + "\n" + fmt_i("internal element number = ", i));
                if (dist > dref * 100.0)
                    die2("Element of very distorted form is found!", "external elemen number = ", p.elem_ext[i],
                         "internal element number = ", i);
                ++k1;
            }
        }
        dave /= (double)k1;
        deqi /= (double)k1;
        p.dmesh_max = dmax; p.dmesh_min = dmin; p.dmesh_ave = dave;
        p.freq_max = p.c / (6.0 * deqi);
        for (i = 0; i < p.n_freq; ++i)
            if (p.freqs[i] > p.freq_max) break;
        if (p.n_freq > i) {
            out << std::endl;
            warn(out, "There are some frequencies higher than the highest allowable frequency!",
                 fmt_i("Number of frequencies outside the range= ", p.n_freq - i) + "\n" +
                     fmt_d("The highest allowable frequency = ", p.freq_max));
        }
        out << p.version << std::endl << p.title << std::endl << std::endl;
        out << "Number of frequency steps ................... = " << p.n_freq << std::endl << std::endl;
        out << "First step .................................. = " << p.first_step << std::endl;
        out << "Number of steps ............................. = " << p.n_freq << std::endl;
        out << "Step increment .............................. = " << p.step_increment << std::endl;
        out << "Highest allowable frequency .................. = " << p.freq_max << std::endl;
        out << "\n\n\n>> B A S I C   P A R A M E T E R S   F O R   B E M <<\n" << std::endl;
        out << "Number of element groups .................... = " << p.n_groups << std::endl;
        out << "Total number of elements .................... = " << NE << std::endl;
        out << "Number of boundary elements ................. = " << p.n_be << std::endl;
        out << "Number of evaluation elements ............... = " << p.n_ev << std::endl;
        out << "Maximum edge length of boundary elements .... = " << dmax << std::endl;
        out << "Average edge length of boundary elements .... = " << dave << std::endl;
        out << "Minimum edge length of boundary elements .... = " << dmin << std::endl << std::endl;
        out << "Total number of nodes ....................... = " << NN << std::endl;
        out << "Number of nodes of the boundary elements .... = " << p.n_nodes_be << std::endl;
        out << "Number of nodes of the evaluation elements .. = " << p.n_nodes_ev << std::endl << std::endl;
        out << "Number of symmetric planes .................. = " << p.n_sym << std::endl << std::endl;
        out << "Number of incident plane waves .............. = " << p.n_plane << std::endl;
        out << "Number of incident spharic waves ............ = " << p.n_point << std::endl << std::endl;
        out << "Sound speed ................................. = " << p.c << std::endl;
        out << "Density of the medium ....................... = " << p.rho << std::endl << std::endl;
        out << "Diameter of the BE-mesh ..................... = " << p.diameter << std::endl;
        if (p.method_bem > 0)
            out << std::endl << "Minimum number of terms in the FMM expansion. = " << p.min_fmm_terms << std::endl;
        out << std::endl;
        out << (p.interior ? "Interior domain problem" : "Exterior domain problem") << std::endl << std::endl;
        out << (p.htf == 1.0 ? "Harmonic time factor = EXP(-i*omega*t)" : "Harmonic time factor = EXP(i*omega*t)")
            << std::endl << std::endl;
        if (p.solver == 0) out << "methodSolver_  = 0: CGS iterative solver" << std::endl;
        else out << "methodSolver_  = 4: Gaussean elimination (direct) solver" << std::endl;
        if (p.solver < 4) {
            if (p.precond == 0) out << "methodPreconditioner_ = 0: incomplete LU-decomposition preconditioner" << std::endl;
            else if (p.precond == 1) out << "methodPreconditioner_ = 1: scaling preconditioner" << std::endl;
            else out << "methodPreconditioner_ = 2: no preconditioner" << std::endl;
            // the GPU path keeps the reference's solution and stopping rule but
            // not its iteration: say so next to the reference's choice
            if (p.precond == 0)
                out << "GPU solver: restarted GMRES (relative residual 1e-9) with a block-Jacobi preconditioner "
                       "(128-unknown blocks, one correction over 1024-unknown windows) in place of CGS with the "
                       "preconditioner above; the direct solver runs when the iteration limit is reached"
                    << std::endl;
            else if (p.precond == 1)
                out << "GPU solver: restarted GMRES (relative residual 1e-9) with the scaling preconditioner above "
                       "in place of CGS; the direct solver runs when the iteration limit is reached"
                    << std::endl;
            else
                out << "GPU solver: restarted GMRES (relative residual 1e-9) without a preconditioner in place of "
                       "CGS; the direct solver runs when the iteration limit is reached"
                    << std::endl;
        } else {
            out << "GPU solver: LU factorisation without pivoting on the GPU (as Tfactor_usy / Tfbelim)" << std::endl;
        }
        const double ell = std::sqrt(p.avg_area);
        out << std::endl << " No.   Freq.   Lambda/L_BE_Mesh  Lambda/L_Element" << std::endl;
        for (i = 0; i < p.n_freq; ++i) {
            const double wavl = p.c / p.freqs[i];
            out << std::setw(3) << i + 1 << " " << std::setw(7) << p.freqs[i] << "   " << std::setw(10)
                << wavl / p.diameter << "        " << std::setw(10) << wavl / ell << std::endl;
        }
        out << std::endl;
    }
}

// NC_FreqCurveInterpolation, NC_EquationSystem.cpp:1964-2009.
static double curve_factor(const Project &p, int id, double frequency) {
    int l1 = -1;
    for (size_t l = 0; l < p.curve_id.size(); ++l)
        if (p.curve_id[l] == id) { l1 = (int)l; break; }
    if (l1 < 0) throw NcExit{"A curve can not be found!\n" + fmt_i("Number of the curve = ", id), 1};
    const auto &f = p.curve_f[l1];
    const auto &fa = p.curve_fac[l1];
    const int np = p.curve_npts[l1];
    if (frequency <= f[0]) return fa[0];
    for (int l = 1; l < np; ++l)
        if (frequency < f[l]) {
            const int l3 = l - 1;
            return fa[l3] + (fa[l] - fa[l3]) / (f[l] - f[l3]) * (frequency - f[l3]);
        }
    return fa[np - 1];
}

// NC_UpdateFreqCurves, NC_EquationSystem.cpp:1815-1961, with the complex
// helpers of NC_TypeDefinition.h (div_i: z / (i y), mul_i: z * (i y)).
static cd div_i(cd z, double y) { return cd(z.imag() / y, -z.real() / y); }
static cd mul_i(cd z, double y) { return cd(-z.imag() * y, z.real() * y); }

void update_freq(const Project &p, double frequency, FreqState &s) {
    const int NE = p.n_elem;
    s.frequency = frequency;
    s.omega = 2.0 * kPI * frequency;
    s.rpfact = p.rho * s.omega * p.htf;
    s.k = s.omega / p.c;
    const double gammfact = s.k * p.htf;
    s.zbval0.assign(4 * (size_t)NE, cd(0.0, 0.0));
    s.zbval1.assign(NE, cd(0.0, 0.0));
    for (int i = 0; i < NE; ++i) {
        if (p.elem_prop[i] == 2) continue;
        for (int j = 0; j < p.elem_nv[i]; ++j) s.zbval0[4 * (size_t)i + j] = p.zbvao0[4 * (size_t)i + j];
        s.zbval1[i] = p.zbvao1[i];
        if (p.ibval[i] < 2) continue;
        int ibg = 2, ied = 5;   // surface admittance; transfer admittances are rejected at input
        for (int j = ibg; j <= ied; ++j) {
            const int ibc = p.ibvcurv[6 * (size_t)i + j];
            if (ibc < 0) continue;
            const double facf = curve_factor(p, ibc, frequency);
            if (j == 2) s.zbval1[i] = cd(s.zbval1[i].real() * facf, s.zbval1[i].imag());
            else if (j == 3) s.zbval1[i] = cd(s.zbval1[i].real(), s.zbval1[i].imag() * facf);
        }
    }
    for (int i = 0; i < NE; ++i) {
        if (p.elem_prop[i] == 2) continue;
        if (p.ibval[i] == 1)
            for (int j = 0; j < p.elem_nv[i]; ++j) s.zbval0[4 * (size_t)i + j] = div_i(s.zbval0[4 * (size_t)i + j], s.rpfact);
        else if (p.ibval[i] == 2)
            s.zbval1[i] = mul_i(s.zbval1[i], gammfact);
    }
    s.zinwav.assign(p.n_plane, cd(0.0, 0.0));
    for (int i = 0; i < p.n_plane; ++i) {
        cd zv = p.plane_amp0[i];
        for (int j = 0; j < 2; ++j) {
            const int ibc = p.plane_curve[2 * i + j];
            if (ibc >= 0) {
                const double facf = curve_factor(p, ibc, frequency);
                zv = j == 0 ? cd(zv.real() * facf, zv.imag()) : cd(zv.real(), zv.imag() * facf);
            }
        }
        s.zinwav[i] = div_i(zv, s.rpfact);
    }
    const int npt = p.n_point > 0 ? p.n_point : 0;
    s.zposoc.assign(npt, cd(0.0, 0.0));
    for (int i = 0; i < npt; ++i) {
        cd zv = p.point_amp0[i];
        for (int j = 0; j < 2; ++j) {
            const int ibc = p.point_curve[2 * i + j];
            if (ibc >= 0) {
                const double facf = curve_factor(p, ibc, frequency);
                zv = j == 0 ? cd(zv.real() * facf, zv.imag()) : cd(zv.real(), zv.imag() * facf);
            }
        }
        s.zposoc[i] = div_i(zv, s.rpfact);
    }
}

namespace {
void put(FILE *f, const char *name, const char *dtype, const void *data, long long count, size_t elsize) {
    char nm[24] = {0}, dt[8] = {0};
    std::strncpy(nm, name, sizeof(nm) - 1);
    std::strncpy(dt, dtype, sizeof(dt) - 1);
    std::fwrite(nm, 1, sizeof(nm), f);
    std::fwrite(dt, 1, sizeof(dt), f);
    std::fwrite(&count, sizeof(count), 1, f);
    if (count > 0) std::fwrite(data, elsize, (size_t)count, f);
}
void put_i(FILE *f, const char *name, const std::vector<int> &v) { put(f, name, "i4", v.data(), (long long)v.size(), 4); }
void put_d(FILE *f, const char *name, const std::vector<double> &v) { put(f, name, "f8", v.data(), (long long)v.size(), 8); }
}  // namespace

void dump_tables(const Project &p, const char *path) {
    FILE *f = std::fopen(path, "wb");
    if (!f) throw NcExit{std::string("cannot write ") + path, 1};
    std::vector<int> sc = {p.n_nodes, p.n_elem, p.n_groups, p.n_nodes_be, p.n_nodes_ev, p.n_be, p.n_ev, p.n_be, p.n_sym};
    put_i(f, "scalars_i", sc);
    std::vector<double> sd = {p.diameter, p.avg_area, p.c, p.rho, p.htf, p.tao};
    put_d(f, "scalars_d", sd);
    put_i(f, "node_ext", p.node_ext);
    put_i(f, "node_class", p.node_class);
    put_d(f, "node_xyz", p.node_xyz);
    put_i(f, "elem_ext", p.elem_ext);
    put_i(f, "elem_nvert", p.elem_nv);
    put_i(f, "elem_prop", p.elem_prop);
    put_i(f, "elem_group", p.elem_group);
    put_i(f, "elem_conn", p.elem_conn);
    std::vector<int> dof(p.n_elem, -1);
    int d = 0;
    for (int e = 0; e < p.n_elem; ++e)
        if (p.elem_prop[e] != 2) dof[e] = d++;
    put_i(f, "elem_dof", dof);
    put_i(f, "elem_ibval", p.ibval);
    put_d(f, "elem_center", p.centel);
    put_d(f, "elem_normals", p.elenor);
    put_d(f, "elem_area", p.areael);
    put_i(f, "group_index", p.group_index);
    put_i(f, "group_count", p.group_count);
    put_i(f, "group_prop", p.group_prop);
    put_d(f, "freqs", p.freqs);
    std::fclose(f);
}

}  // namespace nc
