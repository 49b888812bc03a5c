// wlc_internal.h -- host-side data shared between the set-up code
// (wlc_host.cpp) and the CUDA side (wlc_api.cu, wlc_kernels.cu).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace wlc {

// Harmonic index i <-> (l, m): i = l*l + l + m, m = -l..l
// (basis_sph_create, SPH_mod.f90:192-233).
inline int basis_l(int i) {
    int l = 0;
    while ((l + 1) * (l + 1) <= i) ++l;
    return l;
}
inline int basis_m(int i) {
    int l = basis_l(i);
    return i - l * l - l;
}

// Sparse list of matrix entries (row, col, value).
struct Triplets {
    std::vector<int> row, col;
    std::vector<double> val;
    size_t size() const { return val.size(); }
};

// Everything the k-space operator needs, built once per (L, literal
// semantics) on the host.
struct BasisTables {
    int L = 0, M = 0;
    int real4 = 1;
    // Reference coupling matrices (M x M, row-major): Rx, Ry, Rz
    // (init_array_2dcomp_mod.f90:166-182), Theta basis tensors T1122, T33,
    // T12, T13, T23 (:186-270) and J11, J22, J12, J13, J23 (:276-375).
    std::vector<double> R[3], T[5], J[5];
    // Real-harmonic rotation by +pi/2 about x, per l block, as CSR over
    // output rows (row pointer over all M rows). Xm = Xp^T.
    std::vector<int> xp_ptr, xp_col, xm_ptr, xm_col;
    std::vector<double> xp_val, xm_val;
    // Rz coupling of (l, m) to (l+1, m); 0 for l = L.
    std::vector<double> zoff;
    // Entries where the reference's Rx/Ry/Rz differ from the rotation-
    // covariant operator used by the fast solve (nonzero only under
    // single-precision literal semantics): dR_a = R_a(ref) - R_a(cov).
    Triplets dR[3];
    double max_dR = 0.0;
    // Sparse Theta / J lists with the reference threshold
    // |v| >= Thresh_sprase_matrix (global_parameters.f90:60).
    Triplets Tsp[5], Jsp[5];
};

// Builds all tables; returns false and sets `err` if the host self-check
// of the factorised G(k)^-1 against a dense solve fails.
bool build_basis_tables(int L, int real4, BasisTables& out, std::string& err);

// Literal constants under the chosen semantics.
double lit_c0(int order, int real4);      // BDF1/2/3 diagonal 1, 3/2, 11/6
double lit_third(int real4);              // 1.0/3.0 of the BDF3 history
double lit_thresh(int real4);             // 1.0e-10 sparsity threshold
double lit_kfactor(int n, double d, int real4);  // 2*PI/(SIDE*d), PI of kind SP

// Dense host reference of G(k) (sigma=+1) for the self-check.
void host_dense_G(const BasisTables& t, double c0, double diag_coef, const double k[3], double ds,
                  std::vector<double>& gre, std::vector<double>& gim);

// Host version of the factorised solve used by the device (for the
// self-check): x = G_cov^-1 b, optionally followed by the first-order
// correction for dR.
void host_factored_solve(const BasisTables& t, double c0, double diag_coef, const double k[3],
                         double ds, int sigma, const double* bre, const double* bim, double* xre,
                         double* xim, bool correct);

}  // namespace wlc
