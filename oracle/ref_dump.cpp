// Test infrastructure (oracle only).  Linked into oracle/_ref/NumCalc_dump
// with  -Wl,--wrap=<NC_IterativeSolverCGS>:  every call the reference's
// frequency loop (NC_Main.cpp:836) makes to its CGS solver first lands here.
// When NC_DUMP_DIR is set, this writes
//   tables.bin        parsed mesh and group tables (first call only)
//   step<k>.bin       frequency data, the assembled TBEM matrix (zcoefl,
//                     row-major N x N complex128), the right-hand side
//                     (zrhs) before the solve and the solution after it
// and then calls the reference solver unchanged.
//
// Record format (little endian): name[24] NUL padded, dtype[8] ("f8", "i4",
// "c16"), int64 count, then count elements.

#include "NC_ConstantsVariables.h"
#include "NC_TypeDefinition.h"
#include "NC_Arrays.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

extern int numNodes_, numElements_, numElementGroups_, numRowsOfCoefficientMatrix_;
extern int numNodesOfBoundaryMesh_, numNodesOfEvaluationMesh_;
extern int numElementsOfBoundaryMesh_, numElementsOfEvaluationMesh_;
extern int currentFrequency_, numPointSources_, numIncidentPlaneWaves_;
extern int methodFMM_, methodPreconditioner_, numSymmetricPlanes_;
extern double frequency_, waveNumbers_, rpfact_, diameterBE_, averageElementArea_;
extern double harmonicTimeFactor_, Tao_, speedOfSound_, densityOfMedium_;

namespace {

void put(FILE* f, const char* name, const char* dtype, const void* data,
         long long count, size_t elsize)
{
    char nm[24] = {0}, dt[8] = {0};
    std::strncpy(nm, name, sizeof(nm) - 1);
    std::strncpy(dt, dtype, sizeof(dt) - 1);
    std::fwrite(nm, 1, sizeof(nm), f);
    std::fwrite(dt, 1, sizeof(dt), f);
    std::fwrite(&count, sizeof(count), 1, f);
    if (count > 0) std::fwrite(data, elsize, (size_t)count, f);
}

void put_i(FILE* f, const char* name, const std::vector<int>& v)
{ put(f, name, "i4", v.data(), (long long)v.size(), sizeof(int)); }

void put_d(FILE* f, const char* name, const std::vector<double>& v)
{ put(f, name, "f8", v.data(), (long long)v.size(), sizeof(double)); }

void put_z(FILE* f, const char* name, const Complex* z, long long n)
{
    std::vector<double> v((size_t)(2 * n));
    for (long long i = 0; i < n; ++i) { v[2 * i] = z[i].re(); v[2 * i + 1] = z[i].im(); }
    put(f, name, "c16", v.data(), n, 2 * sizeof(double));
}

std::string path(const char* dir, const std::string& leaf)
{ return std::string(dir) + "/" + leaf; }

void dump_tables(const char* dir)
{
    FILE* f = std::fopen(path(dir, "tables.bin").c_str(), "wb");
    if (!f) { std::fprintf(stderr, "ref_dump: cannot write tables.bin\n"); std::exit(3); }
    std::vector<int> sc = {numNodes_, numElements_, numElementGroups_,
                           numNodesOfBoundaryMesh_, numNodesOfEvaluationMesh_,
                           numElementsOfBoundaryMesh_, numElementsOfEvaluationMesh_,
                           numRowsOfCoefficientMatrix_, numSymmetricPlanes_};
    put_i(f, "scalars_i", sc);
    std::vector<double> sd = {diameterBE_, averageElementArea_, speedOfSound_,
                              densityOfMedium_, harmonicTimeFactor_, Tao_};
    put_d(f, "scalars_d", sd);
    std::vector<int> ext(numNodes_), cls(numNodes_);
    std::vector<double> xyz((size_t)numNodes_ * 3);
    for (int i = 0; i < numNodes_; ++i) {
        ext[i] = extNumbersOfNodes[i];
        cls[i] = isNodeMeshOrEvalNode[i];
        for (int k = 0; k < 3; ++k) xyz[3 * i + k] = nodesCoordinates[i][k];
    }
    put_i(f, "node_ext", ext);
    put_i(f, "node_class", cls);
    put_d(f, "node_xyz", xyz);
    std::vector<int> eext(numElements_), nv(numElements_), prop(numElements_),
        grp(numElements_), conn((size_t)numElements_ * 4, -1), jel(numElements_), ibv(numElements_);
    std::vector<double> cen((size_t)numElements_ * 3), nor((size_t)numElements_ * 15), area(numElements_);
    for (int e = 0; e < numElements_; ++e) {
        eext[e] = extNumbersOfElements[e];
        nv[e] = listNumberNodesPerElement[e];
        prop[e] = listElementProperty[e];
        grp[e] = listElementsElementGroup[e];
        for (int k = 0; k < nv[e]; ++k) conn[4 * e + k] = elementsConnectivity[e][k];
        jel[e] = jelist[e][0];
        ibv[e] = ibval[e];
        for (int k = 0; k < 3; ++k) cen[3 * e + k] = centel[e][k];
        for (int k = 0; k < 15; ++k) nor[15 * e + k] = elenor[e][k];
        area[e] = areael[e];
    }
    put_i(f, "elem_ext", eext);
    put_i(f, "elem_nvert", nv);
    put_i(f, "elem_prop", prop);
    put_i(f, "elem_group", grp);
    put_i(f, "elem_conn", conn);
    put_i(f, "elem_dof", jel);
    put_i(f, "elem_ibval", ibv);
    put_d(f, "elem_center", cen);
    put_d(f, "elem_normals", nor);
    put_d(f, "elem_area", area);
    std::vector<int> gidx(numElementGroups_), gcnt(numElementGroups_), gprop(numElementGroups_);
    for (int g = 0; g < numElementGroups_; ++g) {
        gidx[g] = indexOfElementGroup[g];
        gcnt[g] = numberOfElementsInGroup[g];
        gprop[g] = propertyOfGroup[g];
    }
    put_i(f, "group_index", gidx);
    put_i(f, "group_count", gcnt);
    put_i(f, "group_prop", gprop);
    std::fclose(f);
}

bool tables_written = false;

}  // namespace

extern "C" void __real__Z21NC_IterativeSolverCGSRSt14basic_ofstreamIcSt11char_traitsIcEE(std::ofstream&);

extern "C" void __wrap__Z21NC_IterativeSolverCGSRSt14basic_ofstreamIcSt11char_traitsIcEE(std::ofstream& out)
{
    const char* dir = std::getenv("NC_DUMP_DIR");
    FILE* f = nullptr;
    const int n = numRowsOfCoefficientMatrix_;
    if (dir) {
        if (!tables_written) { dump_tables(dir); tables_written = true; }
        char leaf[64];
        std::snprintf(leaf, sizeof(leaf), "step%d.bin", currentFrequency_ + 1);
        f = std::fopen(path(dir, leaf).c_str(), "wb");
        if (!f) { std::fprintf(stderr, "ref_dump: cannot write %s\n", leaf); std::exit(3); }
        std::vector<double> sd = {frequency_, waveNumbers_, rpfact_};
        put_d(f, "freq_k_rpfact", sd);
        std::vector<int> si = {n, methodFMM_, methodPreconditioner_};
        put_i(f, "n_method_precond", si);
        int nps = numPointSources_ > 0 ? numPointSources_ : 0;
        put_z(f, "zposoc", zposoc, nps);
        put_z(f, "zinwav", zinwav, numIncidentPlaneWaves_);
        std::vector<Complex> b0((size_t)numElements_ * 4), b1(numElements_);
        for (int e = 0; e < numElements_; ++e) {
            for (int k = 0; k < 4; ++k)
                b0[4 * e + k] = (k < listNumberNodesPerElement[e] && listElementProperty[e] != 2)
                                    ? zbval0[e][k] : Complex(0.0, 0.0);
            b1[e] = listElementProperty[e] != 2 ? zbval1[e] : Complex(0.0, 0.0);
        }
        put_z(f, "zbval0", b0.data(), (long long)b0.size());
        put_z(f, "zbval1", b1.data(), (long long)b1.size());
        if (methodFMM_ == 0) put_z(f, "A", zcoefl, (long long)n * n);
        put_z(f, "b", zrhs, n);
        std::fflush(f);
    }
    __real__Z21NC_IterativeSolverCGSRSt14basic_ofstreamIcSt11char_traitsIcEE(out);
    if (f) {
        put_z(f, "x", zrhs, n);
        std::fclose(f);
    }
}
