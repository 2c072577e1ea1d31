// nc_fmm_plan.h - the reference NumCalc's fast-multipole set-up for a
// frequency step, restated for the drop-in's -estimate_ram: the choice
// between traditional, single-level and multilevel FMM BEM, the element
// clusters (and cluster tree), their near and far fields, the expansion
// orders, and the non-zero counts of the FMM matrices that Memory.txt
// reports (mesh2hrtf/NumCalc/src/NC_Addresses.cpp, NC_Main.cpp:391-479 and
// 524-733).  Host code only; the drop-in itself solves every project as a
// dense BEM on the GPU.
#pragma once

#include <ostream>
#include <vector>

#include "nc_project.h"

namespace nc {

struct FmmCluster {
    std::vector<int> elems;   // internal element numbers, in the order the clustering found them
    double center[3] = {0.0, 0.0, 0.0};
    double radius = 0.0;
    int orig = 0;             // the original cluster (itself, or the one this image mirrors)
    int father = -1;          // cluster on the level above (multilevel)
    std::vector<int> near;    // same-level clusters in the near field (itself included)
    int n_far = 0;            // same-level clusters in the far field
    std::vector<int> far;
};

struct FmmLevel {
    // the original clusters, then with symmetry planes their images: for
    // each original in turn its reflections 1 .. n_reflections - 1
    std::vector<FmmCluster> cl;
    int n_orig = 0;
    double r_max = 0.0, r_avg = 0.0, r_min = 0.0;
    int pairs_canceled = 0;   // geometric far pairs closer than the Hankel-argument limit
    int pairs_far = 0;        // geometric far pairs
    int terms = 0, n_theta = 0, n_phi = 0, n_sphere = 0;
};

// Method codes as NumCalc's methodFMM_: 0 traditional BEM, 1 single-level
// FMM, 3 direct multilevel FMM.
class FmmPlan {
public:
    explicit FmmPlan(const Project &p);

    // NC_DeclareArrays (NC_Addresses.cpp:58-287) for frequency step `step`
    // (first == the first step of the run): method and clusters.  Returns
    // false when the previous step's clusters are kept unchanged.
    bool declare(int step, int first, double frequency);
    // Expansion orders and points on the unit sphere for wave number k
    // (NC_Main.cpp:419-479).
    void expansion(double k);
    // The RAM estimate (GB) of NC_Main.cpp:524-733; writes the counts to log
    // as the reference prints them.
    double ram_estimate_gb(std::ostream &log) const;

    int method() const { return method_; }
    int levels() const { return (int)lv_.size(); }
    const FmmLevel &level(int l) const { return lv_[l]; }

private:
    void clusters_of(int lev, const std::vector<std::vector<int>> &groups, FmmLevel &out);
    void merge_small(std::vector<std::vector<int>> &cells) const;
    void cluster_geometry(FmmCluster &c) const;
    void near_far(FmmLevel &L, int lev);
    void reflect(FmmLevel &L, const FmmLevel *father) const;
    int estimate_levels();
    void build_single();
    void build_tree();
    std::vector<std::vector<int>> be_groups() const;

    const Project &p_;
    int n_rows_ = 0;            // unknowns: boundary elements
    double h_arg_min_ = 0.0;    // smallest argument of the spherical Hankel function
    double delta_ = 0.0, eps_ = 1.0e-6;
    double edge1_ = 0.0;        // cluster edge length on level 0 (ClusEdgL1)
    double min_dist_ = 0.0;     // H_Argum_Min / k
    int method_ = 0, prev_method_ = 0, prev_levels_ = 0;
    std::vector<FmmLevel> lv_;
};

}  // namespace nc
