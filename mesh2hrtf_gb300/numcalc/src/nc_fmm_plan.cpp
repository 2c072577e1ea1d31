// nc_fmm_plan.cpp - the reference NumCalc's FMM set-up per frequency step,
// for -estimate_ram (see nc_fmm_plan.h).  Every count and every floating-
// point comparison follows the reference's order of operations so that the
// clusters, their near/far split and the estimate are the reference's own
// (the file is compiled with -ffp-contract=off like the rest of the
// drop-in's host code).
#include "nc_fmm_plan.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <iostream>
#include <sstream>
#include <string>

namespace nc {

namespace {

[[noreturn]] void fail(const std::string &msg, const std::string &s1, double v1, const std::string &s2 = "",
                       double v2 = 0.0, bool two = false) {
    std::ostringstream o;
    o << msg << "\n" << s1 << v1;
    if (two) o << "\n" << s2 << v2;
    throw NcExit{o.str(), 1};
}

double dist3(const double *a, const double *b) {
    return std::sqrt((a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]) + (a[2] - b[2]) * (a[2] - b[2]));
}

// farFieldClusterFactor_ (NC_Main.cpp:84): clusters whose centres are more
// than this times the sum of their radii apart are in each other's far field
const double kFarFactor = 2.0 / std::sqrt(3.0);
constexpr double kSmallCluster = 3.0;   // threshfac1 of NC_CancelSmallClusters
constexpr double kCancelRatio = 0.75;   // thresholrat of NC_DeclareArrays
constexpr int kMaxGaussTheta = 80;      // N_GAUORDER

// spherical-Hankel argument limit per minimum expansion order
// (NC_Main.cpp:347-353)
double hankel_arg_min(int terms) {
    switch (terms) {
    case 5: return 0.0051;
    case 6: return 0.0177;
    case 7: return 0.0445;
    case 8: return 0.0905;
    case 9: return 0.1597;
    case 10: return 0.2547;
    default: return 0.0;
    }
}

// expansion order for a cluster radius (NC_Main.cpp:421-424, 448-452)
int expansion_order(double radius, double k, int min_terms) {
    const double rw = 2.0 * radius * k + 1.8 * std::log10(2.0 * radius * k + kPI);
    int t = (int)rw;
    if (rw - (double)t >= 0.5) ++t;
    if (t < min_terms) t = min_terms;
    return t;
}

}  // namespace

FmmPlan::FmmPlan(const Project &p) : p_(p) {
    n_rows_ = p.n_be;
    h_arg_min_ = hankel_arg_min(p.min_fmm_terms);
    delta_ = p.dmesh_min / 100.0;
}

std::vector<std::vector<int>> FmmPlan::be_groups() const {
    std::vector<std::vector<int>> g;
    for (int i = 0; i < p_.n_groups; ++i) {
        if (p_.group_prop[i] != 0) continue;
        std::vector<int> e;
        for (int j = 0; j < p_.n_elem; ++j)
            if (p_.elem_group[j] == p_.group_index[i]) e.push_back(j);
        g.push_back(std::move(e));
    }
    return g;
}

// centre (mean of the cluster's distinct nodes, in the order the elements
// list them) and radius (farthest node)
void FmmPlan::cluster_geometry(FmmCluster &c) const {
    std::vector<int> nodes;
    for (int e : c.elems)
        for (int a = 0; a < p_.elem_nv[e]; ++a) {
            const int nd = p_.elem_conn[4 * (size_t)e + a];
            bool seen = false;
            for (int q : nodes)
                if (q == nd) { seen = true; break; }
            if (!seen) nodes.push_back(nd);
        }
    double s[3] = {0.0, 0.0, 0.0};
    for (int nd : nodes)
        for (int k = 0; k < 3; ++k) s[k] += p_.node_xyz[3 * (size_t)nd + k];
    for (int k = 0; k < 3; ++k) c.center[k] = s[k] / (double)nodes.size();
    c.radius = 0.0;
    for (int nd : nodes) {
        const double d = dist3(c.center, &p_.node_xyz[3 * (size_t)nd]);
        if (d > c.radius) c.radius = d;
    }
}

// A cell whose radius is under a third of the mean joins the nearest cell
// that is not small (NC_CancelSmallClusters, NC_Addresses.cpp:2077-2244)
void FmmPlan::merge_small(std::vector<std::vector<int>> &cells) const {
    const int n = (int)cells.size();
    std::vector<FmmCluster> g(n);
    double rmin = 1.0e20, ravg = 0.0;
    int used = 0;
    for (int i = 0; i < n; ++i) {
        if (cells[i].empty()) continue;
        g[i].elems = cells[i];
        cluster_geometry(g[i]);
        ravg += g[i].radius;
        ++used;
        if (g[i].radius < rmin) rmin = g[i].radius;
    }
    ravg /= (double)used;
    if (!(ravg > kSmallCluster * rmin)) return;
    std::vector<int> target(n, -1);
    for (int i = 0; i < n; ++i) {
        if (cells[i].empty() || kSmallCluster * g[i].radius >= ravg) continue;
        double dmin = 1.0e20;
        for (int j = 0; j < n; ++j) {
            if (i == j || cells[j].empty() || kSmallCluster * g[j].radius < ravg) continue;
            const double d = dist3(g[i].center, g[j].center);
            if (d < dmin) { dmin = d; target[i] = j; }
        }
    }
    for (int i = 0; i < n; ++i) {
        if (target[i] < 0) continue;
        std::vector<int> &to = cells[target[i]];
        to.insert(to.end(), cells[i].begin(), cells[i].end());
        cells[i].clear();
    }
}

// Clusters of one level: each group (a boundary-element group on level 0, a
// father cluster below) is boxed, the box split into cells of about the
// level's edge length (at most 2 per direction below level 0), elements go
// to the cell holding their centre, small cells are merged
// (NC_GenerateClustersFMM, NC_Addresses.cpp:627-801).
void FmmPlan::clusters_of(int lev, const std::vector<std::vector<int>> &groups, FmmLevel &out) {
    const double edge = lev == 0 ? edge1_ : edge1_ / std::pow(2.0, lev);
    for (size_t gi = 0; gi < groups.size(); ++gi) {
        const std::vector<int> &el = groups[gi];
        double hi[3] = {-1.0e20, -1.0e20, -1.0e20}, lo[3] = {1.0e20, 1.0e20, 1.0e20};
        for (int e : el)
            for (int a = 0; a < p_.elem_nv[e]; ++a) {
                const double *x = &p_.node_xyz[3 * (size_t)p_.elem_conn[4 * (size_t)e + a]];
                for (int k = 0; k < 3; ++k) {
                    if (x[k] > hi[k]) hi[k] = x[k];
                    if (x[k] < lo[k]) lo[k] = x[k];
                }
            }
        int ndiv[3];
        double w[3];
        for (int k = 0; k < 3; ++k) {
            hi[k] += delta_;
            lo[k] -= delta_;
            w[k] = hi[k] - lo[k];
            const double d0 = w[k] / edge;
            int i = (int)d0;
            if (i == 0) i = 1;
            else {
                if (d0 - (double)i > 0.5) ++i;
                if (lev > 0 && i > 2) i = 2;
            }
            ndiv[k] = i;
            w[k] /= (double)i;
        }
        // interval of each element's centre per direction: the first one
        // whose bounds (widened by epsilon) hold it, bounds accumulated
        // from the box's lower corner
        std::vector<int> cell(3 * el.size(), -1);
        for (int k = 0; k < 3; ++k) {
            double d1 = lo[k];
            for (int q = 0; q < ndiv[k]; ++q) {
                const double d0 = d1;
                d1 += w[k];
                for (size_t i = 0; i < el.size(); ++i) {
                    const double c = p_.centel[3 * (size_t)el[i] + k];
                    if (cell[3 * i + k] == -1 && c > d0 - eps_ && c < d1 + eps_) cell[3 * i + k] = q;
                }
            }
        }
        for (size_t i = 0; i < el.size(); ++i)
            for (int k = 0; k < 3; ++k)
                if (cell[3 * i + k] == -1)
                    fail("The interval number of an element is not found!", "number of the element = ",
                         (double)p_.elem_ext[i], "number of the direction = ", (double)k, true);
        std::vector<std::vector<int>> cells;
        for (int a = 0; a < ndiv[0]; ++a)
            for (int b = 0; b < ndiv[1]; ++b)
                for (int c = 0; c < ndiv[2]; ++c) {
                    std::vector<int> m;
                    for (size_t i = 0; i < el.size(); ++i)
                        if (cell[3 * i] == a && cell[3 * i + 1] == b && cell[3 * i + 2] == c) m.push_back(el[i]);
                    cells.push_back(std::move(m));
                }
        merge_small(cells);
        for (auto &m : cells) {
            if (m.empty()) continue;
            FmmCluster c;
            c.elems = std::move(m);
            c.father = lev > 0 ? (int)gi : -1;
            out.cl.push_back(std::move(c));
        }
    }
    out.n_orig = (int)out.cl.size();
    for (int i = 0; i < out.n_orig; ++i) {
        out.cl[i].orig = i;
        cluster_geometry(out.cl[i]);
    }
}

// Images of the level's clusters in the symmetry planes: the same radius,
// the centre mirrored in every plane an odd number of the reflection steps
// cross; an image's father is the same reflection of its original's father
// (NC_ClusterReflectionsSLFMM :508-626, NC_ClusterReflectionsAtLevelMLFMM
// :1317-1475).
void FmmPlan::reflect(FmmLevel &L, const FmmLevel *father) const {
    const int nref = p_.n_reflections;
    if (nref <= 1) return;
    // axis of each reflection step (the order NC_ReflectPointVector uses)
    static const int kStepAxis[8] = {0, 0, 1, 0, 2, 0, 1, 0};
    int first_free = 0, first_plane = 0;
    for (int k = 0; k < 3; ++k)
        if (p_.sym_planes[k] == 0) { first_free = k + 1; break; }
    for (int k = 0; k < 3; ++k)
        if (p_.sym_planes[k] != 0) { first_plane = k; break; }
    const int n = L.n_orig;
    L.cl.reserve((size_t)n * nref);
    for (int icl = 0; icl < n; ++icl) {
        int crossings[3] = {0, 0, 0};
        for (int kref = 1; kref < nref; ++kref) {
            int dir;
            if (nref == 8) dir = kStepAxis[kref];
            else if (nref == 4) {
                dir = first_free + kStepAxis[kref];
                if (dir >= 3) dir -= 3;
            } else dir = first_plane;
            ++crossings[dir];
            const FmmCluster &o = L.cl[icl];
            FmmCluster c;
            c.elems = o.elems;
            c.radius = o.radius;
            c.orig = icl;
            for (int k = 0; k < 3; ++k)
                c.center[k] = crossings[k] % 2 ? 2.0 * p_.sym_coords[k] - o.center[k] : o.center[k];
            if (father) c.father = father->n_orig + (nref - 1) * o.father + (kref - 1);
            L.cl.push_back(std::move(c));
        }
    }
}

// radii statistics and the near/far split of one level
// (NC_ComputeClusterArraysSLFMM :437-490, NC_GenerateClusterArrayAtLevelMLFMM
// :1044-1100)
void FmmPlan::near_far(FmmLevel &L, int) {
    const int n = (int)L.cl.size();
    L.r_max = L.r_avg = 0.0;
    L.r_min = 1.0e40;
    for (int i = 0; i < L.n_orig; ++i) {
        const double r = L.cl[i].radius;
        if (r > L.r_max) L.r_max = r;
        if (r < L.r_min) L.r_min = r;
        L.r_avg += r;
    }
    L.r_avg /= (double)L.n_orig;
    L.pairs_canceled = L.pairs_far = 0;
    std::vector<char> far((size_t)n * n, 0);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < i; ++j) {
            const double d = dist3(L.cl[i].center, L.cl[j].center);
            const double r = L.cl[i].radius + L.cl[j].radius;
            if (d > kFarFactor * r) {
                if (d > min_dist_) far[(size_t)i * n + j] = far[(size_t)j * n + i] = 1;
                else ++L.pairs_canceled;
                ++L.pairs_far;
            }
        }
    for (int i = 0; i < n; ++i) {
        FmmCluster &c = L.cl[i];
        c.near.clear();
        c.far.clear();
        for (int j = 0; j < n; ++j) (far[(size_t)i * n + j] ? c.far : c.near).push_back(j);
        c.n_far = (int)c.far.size();
    }
}

// number of tree levels and the level-0 edge length
// (NC_EstimateNumLevelsMLFMM, NC_Addresses.cpp:804-845)
int FmmPlan::estimate_levels() {
    const double ele = std::sqrt(p_.avg_area), d_min = 25.0;
    double nroot = std::sqrt((double)p_.n_be) * 0.9;
    if (nroot < d_min) nroot = d_min;
    const double l_min = std::sqrt(d_min) * ele;
    if (p_.clus_edge <= 0.0) {
        const double nels = (double)p_.n_be / nroot;
        edge1_ = std::sqrt(nels) * ele;
    } else {
        edge1_ = p_.clus_edge;
        if (edge1_ < l_min)
            fail("Inputed value of cluster diameter for level 0 is too small!",
                 "Inputed value of cluster diameter for level 0 = ", edge1_,
                 "Smallst allowable value of cluster diameter for level 0 = ", l_min, true);
    }
    const double d = std::log10(edge1_ / l_min) / std::log10(2.0);
    int n = (int)d;
    if (d - (double)n > 0.5) ++n;
    ++n;
    if (n <= 0) n = 1;
    return n;
}

void FmmPlan::build_single() {
    const double nels = std::sqrt((double)p_.n_be);
    if (p_.clus_edge <= 0.0) {
        edge1_ = std::sqrt(nels * p_.avg_area);
    } else {
        edge1_ = p_.clus_edge;
        if (edge1_ < std::sqrt(4.0 * p_.avg_area))
            fail("The read cluster diameter is too small!", "Inputed value of cluster diameter = ", edge1_,
                 "The smallst allowable value       = ", std::sqrt(4.0 * p_.avg_area), true);
    }
    lv_.assign(1, FmmLevel());
    clusters_of(0, be_groups(), lv_[0]);
    reflect(lv_[0], nullptr);
    near_far(lv_[0], 0);
}

void FmmPlan::build_tree() {
    const int levels = (int)lv_.size();
    for (int l = 0; l < levels; ++l) {
        std::vector<std::vector<int>> groups;
        if (l == 0) groups = be_groups();
        else
            for (int i = 0; i < lv_[l - 1].n_orig; ++i) groups.push_back(lv_[l - 1].cl[i].elems);
        clusters_of(l, groups, lv_[l]);
        reflect(lv_[l], l > 0 ? &lv_[l - 1] : nullptr);
        near_far(lv_[l], l);
    }
}

bool FmmPlan::declare(int step, int first, double frequency) {
    const double omega = 2.0 * kPI * frequency;
    const double k = omega / p_.c;
    const double wavelength = p_.c / frequency;
    min_dist_ = h_arg_min_ / k;
    const double ratio = wavelength / p_.diameter;
    int method = method_, levels = 1;
    if (p_.method_bem == 0 || ratio > 80.0) {
        method = 0;
    } else if (p_.method_bem == 1) {
        method = 1;
    } else if (ratio > 1.0) {
        method = 1;
    } else {
        levels = estimate_levels();
        if (levels == 1) method = 1;
        else if (p_.method_bem == 4) method = 3;
        if (levels > 10) fail("numClusterLevels_ must <= 10!", "numClusterLevels_ = ", levels);
    }
    bool changed = true;
    for (;;) {
        if (step > first) {
            if (method == prev_method_ && levels == prev_levels_) changed = false;
            int canceled = 0;
            for (const FmmLevel &L : lv_) canceled += L.pairs_canceled;
            if (!changed && canceled == 0) {
                method_ = method;
                return false;
            }
        }
        lv_.clear();
        if (method == 1) build_single();
        else if (method >= 2) {
            lv_.assign(levels, FmmLevel());
            build_tree();
        }
        prev_method_ = method;
        prev_levels_ = levels;
        // too many cluster pairs cancelled (closer than the Hankel limit):
        // fall back to the next simpler method
        bool again = false;
        for (size_t l = 0; l < lv_.size() && !again; ++l) {
            const FmmLevel &L = lv_[l];
            const double r = L.pairs_canceled > 0 ? (double)L.pairs_canceled / (double)L.pairs_far : 0.0;
            if (method == 1 && l > 0) break;
            if (r > kCancelRatio) {
                if (method == 1) {
                    if (n_rows_ >= 20000)
                        fail("Frquency is too low, the single level FMBEM can not be used! Also, the number of "
                             "elements for the traditioal BEM is limited to 20000 Elements (~ 6.4Gb). Stopping "
                             "NumCalc",
                             "Frequency = ", frequency);
                    method = 0;
                } else {
                    if (n_rows_ >= 50000)
                        fail("Frquency is too low, the multilevel FMBEM can not be used!", "Frequency = ", frequency);
                    method = 1;
                }
                levels = 1;
                changed = true;
                again = true;
            }
        }
        if (!again) break;
    }
    method_ = method;
    return true;
}

void FmmPlan::expansion(double k) {
    for (FmmLevel &L : lv_) {
        L.terms = expansion_order(L.r_max, k, p_.min_fmm_terms);
        L.n_theta = L.terms;
        if (L.n_theta > kMaxGaussTheta)
            fail("Too many integral points in the theta-direction!", "Number of integration points = ",
                 L.n_theta, "Maximum allowable number of integration points = ", kMaxGaussTheta, true);
        L.n_phi = 2 * L.n_theta;
        L.n_sphere = L.n_theta * L.n_phi;
    }
}

double FmmPlan::ram_estimate_gb(std::ostream &log) const {
    // unsigned 32-bit counts and int products, as the reference keeps them
    using u32 = uint32_t;
    const u32 N = (u32)n_rows_;
    u32 nint = 0, ncmplx = N;   // the right-hand side
    // near-field entries: each original cluster's elements times the
    // elements of the original clusters whose images or selves are near it
    auto nearfield = [&](const FmmLevel &L) {
        u32 nnz = 0;
        std::vector<char> seen(L.n_orig);
        for (int i = 0; i < L.n_orig; ++i) {
            std::fill(seen.begin(), seen.end(), 0);
            for (int j : L.cl[i].near) seen[L.cl[j].orig] = 1;
            u32 nij = 0;
            for (int j = 0; j < L.n_orig; ++j)
                if (seen[j]) nij += (u32)L.cl[j].elems.size();
            nnz += (u32)L.cl[i].elems.size() * nij;
        }
        return nnz;
    };
    auto all_elems = [](const FmmLevel &L) {
        u32 n = 0;
        for (const FmmCluster &c : L.cl) n += (u32)c.elems.size();
        return n;
    };
    if (method_ == 0) {
        log << "TBEM: \n";
        log << "Number of entries right hand side: " << ncmplx << "\n";
        log << "Number of Matrix entries: " << ncmplx * ncmplx << "\n";
        ncmplx += N * N;
    } else if (method_ == 1) {
        const FmmLevel &L = lv_[0];
        const u32 ns = (u32)L.n_sphere, nall = (u32)L.cl.size(), norig = (u32)L.n_orig;
        ncmplx += ns * 2u;
        u32 nnz = nearfield(L);
        log << "SLFMM:\n";
        log << "Nearfield: " << (int)nnz << "\n";
        nint += nnz + N + 1u;
        ncmplx += nnz;
        nnz = all_elems(L) * ns;
        ncmplx += nnz;
        nint += nnz + ns * nall + 1u;
        log << "T Matrix: " << (int)nnz << "\n";
        nnz = 0;
        for (int i = 0; i < L.n_orig; ++i) nnz += (u32)L.cl[i].n_far;
        nnz *= ns;
        nint += nnz + norig * ns;
        ncmplx += nnz;
        log << "D Matrix: " << (int)nnz << "\n";
        nnz = N * ns;
        nint += nnz + N + 1u;
        ncmplx += nnz;
        log << "S Matrix: " << (int)nnz << "\n";
    } else {
        const FmmLevel &top = lv_.back();
        ncmplx += (u32)top.n_sphere * 2u;
        u32 nnz = nearfield(top);
        nint += nnz + N + 1u;
        ncmplx += nnz;
        log << "MLFMM: \n";
        log << "Nearfield " << (int)nnz << "\n";
        for (size_t l = 0; l < lv_.size(); ++l) {
            const FmmLevel &L = lv_[l];
            nnz = all_elems(L) * (u32)L.n_sphere;
            log << "Tmatrix level " << l << ": " << (int)nnz << "\n";
            nint += nnz + (u32)L.cl.size() * (u32)L.n_sphere + 1u;
            ncmplx += nnz;
        }
        for (size_t l = 0; l < lv_.size(); ++l) {
            const FmmLevel &L = lv_[l];
            nnz = 0;
            if (l == 0) {
                for (int i = 0; i < L.n_orig; ++i) nnz += (u32)L.cl[i].n_far * (u32)L.n_sphere;
            } else {
                // far clusters whose father is in the near field of the
                // cluster's own father (the interactions this level adds)
                const FmmLevel &F = lv_[l - 1];
                const size_t nf = F.cl.size();
                std::vector<char> near((size_t)F.n_orig * nf, 0);
                for (int i = 0; i < F.n_orig; ++i)
                    for (int j : F.cl[i].near) near[(size_t)i * nf + j] = 1;
                for (int i = 0; i < L.n_orig; ++i) {
                    const FmmCluster &c = L.cl[i];
                    u32 m = 0;
                    for (int j : c.far)
                        if (near[(size_t)c.father * nf + L.cl[j].father]) ++m;
                    nnz += m * (u32)L.n_sphere;
                }
            }
            log << "D Matrix level " << l << ": " << (int)nnz << "\n";
            nint += nnz + (u32)L.n_orig * (u32)L.n_sphere + 1u;
            ncmplx += nnz;
        }
        for (size_t l = 0; l < lv_.size(); ++l) {
            nnz = N * (u32)lv_[l].n_sphere;
            nint += nnz + N + 1u;
            ncmplx += nnz;
            log << "S Matrix level " << l << ": " << (int)nnz << "\n";
        }
    }
    log << "Total Nr. of Integers: " << nint << "\n";
    log << "Total Nr. of Cmplxdble: " << ncmplx << "\n";
    const double gb = (double)((size_t)nint * sizeof(int) + (size_t)ncmplx * 16) / 1000.0 / 1000.0 / 1000.0;
    log << "RAM Estimation: " << gb << " GByte\n";
    return gb;
}

}  // namespace nc
