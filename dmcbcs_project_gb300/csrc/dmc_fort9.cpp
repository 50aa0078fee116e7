// Walker-configuration files in the reference's fort.9 format.
//
// Write (dmcbcs.f90:548-567), walkers in pop order (the top of the stack
// first):
//     write (9,'(i10,f15.8)') nt, tau
//     per walker:  write (9,'(6e15.7)') x            3*npart values, 6 per record
//                  write (9,'(e15.7,2e25.15)') weight, psil, psigl
//                  write (9,'(i20,2e15.7)') irn      only the i20 field is output
// Read (dmcbcs.f90:254-258,283-294), walkers pushed in file order:
//     read (9,'(i10,f15.8)') n1, tau0
//     per walker:  read (9,'(6e15.7)') x
//                  read (9,'(e15.7,2e25.15)') weight, psil0, psigl0
//                  read (9,'(i20)') irn
// The generator pairsconfig.f90:25-37 writes the same layout with an (i10)
// header and a weight-only second record; blank fields read as zero, as
// Fortran formatted input does.
//
// Host code only: no CUDA call.  The edit descriptors are implemented here:
// Ew.d output is [-]0.<d digits>E+ee (the letter dropped for |exponent| >
// 99), right-justified in w columns; input takes a fixed-width field,
// ignores blanks, accepts E, D or a signed exponent without a letter, and
// applies the implied decimal point when the field has none.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/dmcbcs_gpu.h"

#include "dmc_text.h"

namespace dmc {

// Fortran Ew.d output
std::string fortran_e(double v, int w, int d)
{
    std::string body;
    if (!std::isfinite(v)) {
        body = std::isnan(v) ? "NaN" : (v > 0 ? "Infinity" : "-Infinity");
    } else if (v == 0.0) {
        body = std::string(std::signbit(v) ? "-0." : "0.") + std::string(d, '0') + "E+00";
    } else {
        // d significant digits: printf's %.{d-1}e gives m.mmm e x, which is
        // 0.mmmm e (x+1)
        char buf[64];
        std::snprintf(buf, sizeof buf, "%.*e", d - 1, std::fabs(v));
        std::string s(buf);
        const size_t epos = s.find('e');
        std::string mant = s.substr(0, epos);
        const int ex = std::atoi(s.c_str() + epos + 1) + 1;
        std::string digits;
        for (char ch : mant)
            if (ch != '.') digits += ch;
        char eb[16];
        if (std::abs(ex) <= 99)
            std::snprintf(eb, sizeof eb, "E%c%02d", ex < 0 ? '-' : '+', std::abs(ex));
        else
            std::snprintf(eb, sizeof eb, "%c%03d", ex < 0 ? '-' : '+', std::abs(ex));
        body = std::string(v < 0 ? "-" : "") + "0." + digits + eb;
    }
    if ((int)body.size() > w) return std::string(w, '*');
    return std::string(w - body.size(), ' ') + body;
}

}  // namespace dmc

namespace {

using dmc::fortran_e;

// Fortran Ew.d / Fw.d input of one fixed-width field (blank = 0)
bool read_real(const std::string& field, int d, double& out)
{
    std::string s;
    for (char ch : field)
        if (ch != ' ' && ch != '\t' && ch != '\r' && ch != '\n') s += ch;
    if (s.empty()) {
        out = 0.0;
        return true;
    }
    for (auto& ch : s)
        if (ch == 'd' || ch == 'D' || ch == 'e' || ch == 'q' || ch == 'Q') ch = 'E';
    // a sign after the first mantissa character starts an exponent without a letter
    if (s.find('E') == std::string::npos)
        for (size_t i = 1; i < s.size(); ++i)
            if ((s[i] == '+' || s[i] == '-') && s[i - 1] != 'E') {
                s.insert(i, "E");
                break;
            }
    const size_t epos = s.find('E');
    std::string mant = epos == std::string::npos ? s : s.substr(0, epos);
    std::string expo = epos == std::string::npos ? "" : s.substr(epos + 1);
    if (mant.find('.') == std::string::npos) {
        // implied decimal point: the last d digits are the fraction
        std::string sign;
        if (!mant.empty() && (mant[0] == '+' || mant[0] == '-')) {
            sign = mant.substr(0, 1);
            mant = mant.substr(1);
        }
        if (d > 0) {
            if ((int)mant.size() < d) mant = std::string(d - mant.size(), '0') + mant;
            mant = mant.substr(0, mant.size() - d) + "." + mant.substr(mant.size() - d);
        }
        mant = sign + mant;
    }
    std::string t = mant + (expo.empty() ? "" : "E" + expo);
    char* end = nullptr;
    out = std::strtod(t.c_str(), &end);
    return end && *end == '\0';
}

bool read_int(const std::string& field, int64_t& out)
{
    std::string s;
    for (char ch : field)
        if (ch != ' ' && ch != '\t' && ch != '\r' && ch != '\n') s += ch;
    if (s.empty()) {
        out = 0;
        return true;
    }
    char* end = nullptr;
    out = std::strtoll(s.c_str(), &end, 10);
    return end && *end == '\0';
}

std::string field_at(const std::string& line, size_t pos, size_t w)
{
    if (pos >= line.size()) return std::string();
    return line.substr(pos, w);
}

struct LineReader {
    FILE* f;
    bool next(std::string& line)
    {
        line.clear();
        int ch;
        bool any = false;
        while ((ch = std::fgetc(f)) != EOF) {
            any = true;
            if (ch == '\n') break;
            line += (char)ch;
        }
        if (!line.empty() && line.back() == '\r') line.pop_back();
        return any;
    }
};

}  // namespace

extern "C" {

int dmc_fort9_write(const char* path, int npart, int n, const double* x, const double* weight, const double* psil,
                    const double* psigl, const int64_t* irn, double tau)
{
    if (!path || npart < 1 || n < 0 || (n > 0 && (!x || !weight || !psil || !psigl || !irn))) return DMC_ERR_INVALID;
    FILE* f = std::fopen(path, "w");
    if (!f) return DMC_ERR_INVALID;
    const int n3 = 3 * npart;
    std::fprintf(f, "%10d%15.8f\n", n, tau);
    for (int k = 0; k < n; ++k) {
        const double* xk = x + (size_t)k * n3;
        for (int e = 0; e < n3; ++e) {
            std::fputs(fortran_e(xk[e], 15, 7).c_str(), f);
            if (e % 6 == 5 || e == n3 - 1) std::fputc('\n', f);
        }
        std::fputs(fortran_e(weight[k], 15, 7).c_str(), f);
        std::fputs(fortran_e(psil[k], 25, 15).c_str(), f);
        std::fputs(fortran_e(psigl[k], 25, 15).c_str(), f);
        std::fputc('\n', f);
        std::fprintf(f, "%20lld\n", (long long)irn[k]);
    }
    const bool ok = std::ferror(f) == 0;
    std::fclose(f);
    return ok ? DMC_OK : DMC_ERR_INVALID;
}

int dmc_fort9_read(const char* path, int npart, int cap, double* x, double* weight, double* psil0, double* psigl0,
                   int64_t* irn, int* n, double* tau)
{
    if (!path || npart < 1 || cap < 0 || !n) return DMC_ERR_INVALID;
    FILE* f = std::fopen(path, "r");
    if (!f) return DMC_ERR_INVALID;
    LineReader rd{f};
    std::string line;
    int rc = DMC_OK;
    int64_t n1 = 0;
    double t0 = 0.0;
    if (!rd.next(line) || !read_int(field_at(line, 0, 10), n1) || !read_real(field_at(line, 10, 15), 8, t0) || n1 < 0) {
        std::fclose(f);
        return DMC_ERR_INVALID;
    }
    *n = (int)n1;
    if (tau) *tau = t0;
    if (n1 == 0) {
        std::fclose(f);
        return DMC_OK;
    }
    if (n1 > cap || !x || !irn) {
        std::fclose(f);
        return n1 > cap ? DMC_ERR_OVERFLOW : DMC_ERR_INVALID;
    }
    const int n3 = 3 * npart;
    for (int64_t k = 0; k < n1 && rc == DMC_OK; ++k) {
        double* xk = x + (size_t)k * n3;
        for (int e0 = 0; e0 < n3 && rc == DMC_OK; e0 += 6) {
            if (!rd.next(line)) {
                rc = DMC_ERR_INVALID;
                break;
            }
            for (int e = e0; e < std::min(n3, e0 + 6); ++e)
                if (!read_real(field_at(line, 15 * (e - e0), 15), 7, xk[e])) rc = DMC_ERR_INVALID;
        }
        if (rc != DMC_OK) break;
        double w = 0.0, p0 = 0.0, pg0 = 0.0;
        if (!rd.next(line) || !read_real(field_at(line, 0, 15), 7, w) || !read_real(field_at(line, 15, 25), 15, p0) ||
            !read_real(field_at(line, 40, 25), 15, pg0)) {
            rc = DMC_ERR_INVALID;
            break;
        }
        if (weight) weight[k] = w;
        if (psil0) psil0[k] = p0;
        if (psigl0) psigl0[k] = pg0;
        int64_t r = 0;
        if (!rd.next(line) || !read_int(field_at(line, 0, 20), r)) {
            rc = DMC_ERR_INVALID;
            break;
        }
        irn[k] = r;
    }
    std::fclose(f);
    return rc;
}

}  // extern "C"
