// wlc_io.cpp -- the reference's field / density / free-energy files, so that
// a run can start from the Fortran code's output and the other way round.
// Host-only C functions on host arrays (no context, no device work).
//
//   W<rank>.dat       K  W_A(K)  W_B(K)  [W_C(K)]          (W_dump / readW,
//                     SCFT_dump.f90:296-300, init_array_2dcomp_mod.f90:1088-1093)
//   M_OP<rank>.dat    3 lines per point: Lx Ly Lz M(a,0) M(a,1) M(a,2)
//                     (SCFT_dump.f90:302-308, init_array_2dcomp_mod.f90:1095-1102)
//   RHO_total.dat     '(3f10.6,3f12.8)' x y z phi_A phi_B phi_C, z outermost,
//                     x innermost (SCFT_dump.f90:116-127)
//   FreeEG.dat        n_iter F lnQ (F + lnQ) (F - F_FH) / n_iter box "FE-FH" (F - F_FH)
//                     (SCFT_dump.f90:40-42); error.dat n_iter errors (:36-38)
//
// List-directed files are written with 17 significant digits and read with
// any whitespace or comma separation and Fortran D exponents.
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "wlc.h"

namespace {

struct File {
    FILE* f = nullptr;
    File(const char* path, const char* mode) : f(path ? std::fopen(path, mode) : nullptr) {}
    ~File() {
        if (f) std::fclose(f);
    }
};

// next line split into numbers (Fortran list-directed: blanks or commas,
// D or d exponents); false at end of file
bool read_numbers(FILE* f, std::vector<double>& out) {
    out.clear();
    std::string line;
    int ch;
    bool any = false;
    while ((ch = std::fgetc(f)) != EOF) {
        any = true;
        if (ch == '\n') break;
        line.push_back((char)ch);
    }
    if (!any) return false;
    for (char& c : line) {
        if (c == 'D' || c == 'd') c = 'E';
        if (c == ',') c = ' ';
    }
    const char* p = line.c_str();
    while (*p) {
        while (*p && std::isspace((unsigned char)*p)) ++p;
        if (!*p) break;
        char* end = nullptr;
        const double v = std::strtod(p, &end);
        if (end == p) break;  // a word (e.g. a label): stop at it
        out.push_back(v);
        p = end;
    }
    return true;
}

}  // namespace

extern "C" int wlc_io_write_w(const char* path, const double* w, int64_t nr) {
    if (!w || nr <= 0) return WLC_E_PARAM;
    File f(path, "w");
    if (!f.f) return WLC_E_IO;
    for (int64_t r = 0; r < nr; ++r)
        if (std::fprintf(f.f, "%12lld %25.17E %25.17E %25.17E\n", (long long)r, w[r], w[nr + r], w[2 * nr + r]) < 0)
            return WLC_E_IO;
    return WLC_OK;
}

extern "C" int wlc_io_read_w(const char* path, double* w, int64_t nr) {
    if (!w || nr <= 0) return WLC_E_PARAM;
    File f(path, "r");
    if (!f.f) return WLC_E_IO;
    std::vector<double> v;
    for (int64_t r = 0; r < nr; ++r) {
        do {
            if (!read_numbers(f.f, v)) return WLC_E_IO;
        } while (v.empty());
        if (v.size() < 3) return WLC_E_IO;
        w[r] = v[1];
        w[nr + r] = v[2];
        w[2 * nr + r] = v.size() >= 4 ? v[3] : 0.0;  // two-block file: w_C = 0
    }
    return WLC_OK;
}

extern "C" int wlc_io_write_mop(const char* path, const double* m_op, int64_t nr, const double* box) {
    if (!m_op || !box || nr <= 0) return WLC_E_PARAM;
    File f(path, "w");
    if (!f.f) return WLC_E_IO;
    for (int64_t r = 0; r < nr; ++r)
        for (int a = 0; a < 3; ++a)
            if (std::fprintf(f.f, "%25.17E %25.17E %25.17E %25.17E %25.17E %25.17E\n", box[0], box[1], box[2],
                             m_op[r + nr * (a + 0)], m_op[r + nr * (a + 3)], m_op[r + nr * (a + 6)]) < 0)
                return WLC_E_IO;
    return WLC_OK;
}

extern "C" int wlc_io_read_mop(const char* path, double* m_op, int64_t nr) {
    if (!m_op || nr <= 0) return WLC_E_PARAM;
    File f(path, "r");
    if (!f.f) return WLC_E_IO;
    std::vector<double> v;
    for (int64_t r = 0; r < nr; ++r)
        for (int a = 0; a < 3; ++a) {
            do {
                if (!read_numbers(f.f, v)) return WLC_E_IO;
            } while (v.empty());
            if (v.size() < 6) return WLC_E_IO;
            for (int b = 0; b < 3; ++b) m_op[r + nr * (a + 3 * b)] = v[3 + b];
        }
    return WLC_OK;
}

extern "C" int wlc_io_write_rho(const char* path, const double* phi, const int32_t* n, const double* dx) {
    if (!phi || !n || !dx || n[0] <= 0 || n[1] <= 0 || n[2] <= 0) return WLC_E_PARAM;
    File f(path, "w");
    if (!f.f) return WLC_E_IO;
    const int64_t nr = (int64_t)n[0] * n[1] * n[2];
    for (int z = 0; z < n[2]; ++z)
        for (int y = 0; y < n[1]; ++y)
            for (int x = 0; x < n[0]; ++x) {
                const int64_t r = x + (int64_t)n[0] * (y + (int64_t)n[1] * z);
                if (std::fprintf(f.f, "%10.6f%10.6f%10.6f%12.8f%12.8f%12.8f\n", x * dx[0], y * dx[1], z * dx[2], phi[r],
                                 phi[nr + r], phi[2 * nr + r]) < 0)
                    return WLC_E_IO;
            }
    return WLC_OK;
}

extern "C" int wlc_io_append_free_energy(const char* path, int32_t n_iter, double fe, double lnq, double box,
                                         const double* chi, const int32_t* ns, int32_t nmax) {
    if (!chi || !ns || nmax <= 0) return WLC_E_PARAM;
    File f(path, "a");
    if (!f.f) return WLC_E_IO;
    // Flory-Huggins energy of the homogeneous melt, sum_{K<J} chi_KJ f_K f_J
    // (the reference's NXAB fa fb for two blocks); chi = (AB, AC, BC)
    const double fa = (double)ns[0] / nmax, fb = (double)ns[1] / nmax, fc = (double)ns[2] / nmax;
    const double fh = chi[0] * fa * fb + chi[1] * fa * fc + chi[2] * fb * fc;
    if (std::fprintf(f.f, "%12d %25.17E %25.17E %25.17E %25.17E\n", n_iter, fe, lnq, fe + lnq, fe - fh) < 0 ||
        std::fprintf(f.f, "%12d %25.17E FE-FH %25.17E\n", n_iter, box, fe - fh) < 0)
        return WLC_E_IO;
    return WLC_OK;
}

extern "C" int wlc_io_append_errors(const char* path, int32_t n_iter, const double* err, int32_t nerr) {
    if (!err || nerr < 1) return WLC_E_PARAM;
    File f(path, "a");
    if (!f.f) return WLC_E_IO;
    std::fprintf(f.f, "%12d", n_iter);
    for (int i = 0; i < nerr; ++i) std::fprintf(f.f, " %25.17E", err[i]);
    if (std::fprintf(f.f, "\n") < 0) return WLC_E_IO;
    return WLC_OK;
}
