// Host-side TableReader: reads one '#$NAME'-tagged section of an Object-MD
// table file and computes its spline coefficients in FP64 with the
// reference's own algorithm (treader.cpp:37-136), so the device only ever
// sees the coefficients the reference would use.
#include <cmath>
#include <fstream>
#include <map>
#include <sstream>

#include "omdg_internal.h"

namespace omdg {

// treader.cpp:83-136 and param.cpp:106-136 (read_pseudo): every token after
// '#$NAME' on its lines goes into one flat list, up to the '#$NAME --' line;
// a key's value is the token after its first occurrence (param.cpp:165-171,
// 218-223), so a line such as '#$EDENS eldens Spacing 1e-3' still gives
// Spacing.  Then NumberOfData values follow the '--' line.
int table_load(const std::string& file, const std::string& name, HostTable& t, std::string& err) {
    std::ifstream fl(file.c_str());
    if (!fl.good()) {
        err = "can not open table file " + file;
        return OMDG_EFILE;
    }
    std::string tag = "#$" + name;
    std::vector<std::string> spar;
    std::string line;
    bool found = false;
    while (std::getline(fl, line)) {
        std::istringstream ss(line);
        std::string s, tok;
        ss >> s >> tok;
        if (s != tag) continue;
        if (tok == "--") {
            found = true;
            break;
        }
        if (!tok.empty()) spar.push_back(tok);
        while (ss >> tok) spar.push_back(tok);
    }
    if (!found) {
        err = "can not find table " + name + "@" + file;
        return OMDG_EFILE;
    }
    auto exists = [&](const char* k) {
        for (const std::string& v : spar)
            if (v == k) return true;
        return false;
    };
    // the token after the key's first occurrence (ParamHandler::double_value)
    auto value_of = [&](const char* k, std::string& out) -> bool {
        for (size_t i = 0; i < spar.size(); i++)
            if (spar[i] == k) {
                if (i + 1 >= spar.size()) return false;
                out = spar[i + 1];
                return true;
            }
        return false;
    };
    auto num = [&](const char* k, double def, bool required, double& out) -> bool {
        std::string v;
        if (!value_of(k, v)) {
            if (required) return false;
            out = def;
            return true;
        }
        std::istringstream vs(v);  // as_double (omdtool.cpp:98-104)
        if (v == "inf") out = 1.79769313486231570815e+308;
        else if (v == "-inf") out = -1.79769313486231570815e+308;
        else if (!(vs >> out)) return false;
        return true;
    };
    double nd = 0, dr = 0, off = 0;
    if (!num("NumberOfData", 0, true, nd) || !num("Spacing", 0, true, dr)) {
        err = "table " + name + "@" + file + " lacks NumberOfData/Spacing";
        return OMDG_EFILE;
    }
    num("Offset", 0.0, false, off);
    t.file = file;
    t.name = name;
    t.n = (int)nd;
    t.dr = dr;
    t.off = off;
    t.rmult = false;
    std::string fmt;
    if (value_of("Format", fmt)) {
        if (fmt == "RMULT") t.rmult = true;
        else if (fmt != "PLAIN") {
            err = "unsupported format " + fmt;
            return OMDG_EFILE;
        }
    }
    t.allow_lo = exists("OutOfRangeLower");
    t.allow_hi = exists("OutOfRangeUpper");
    t.has_constant = exists("Constant");
    num("Constant", 0.0, false, t.constant);
    num("OutOfRangeLower", 0.0, false, t.out_lo);
    num("OutOfRangeUpper", 0.0, false, t.out_hi);
    if (t.n < 4 || !(t.dr > 0)) {
        err = "table " + name + "@" + file + " too small";
        return OMDG_EFILE;
    }
    t.d.assign(t.n, 0.0);
    for (int i = 0; i < t.n; i++) {
        if (!(fl >> t.d[i])) {
            err = "table " + name + "@" + file + " has fewer than NumberOfData values";
            return OMDG_EFILE;
        }
    }
    table_coef(t);
    return OMDG_OK;
}

// treader.cpp:37-64, same operation order (the tridiagonal system with end
// rows b=5 and S[0]=S[1], S[n+1]=S[n]).
void table_coef(HostTable& t) {
    int nd = t.n;
    int n = nd - 2;
    std::vector<double> b(n), d(n), S(nd);
    double dr = t.dr;
    t.a.assign(nd, 0.0);
    t.b.assign(nd, 0.0);
    t.c.assign(nd, 0.0);
    for (int i = 1; i < n + 1; i++) d[i - 1] = t.d[i + 1] - 2.0 * t.d[i] + t.d[i - 1];
    for (int i = 1; i < n - 1; i++) b[i] = 4.0;
    b[0] = b[n - 1] = 5.0;
    for (int k = 1; k < n; k++) {
        double m = 1.0 / b[k - 1];
        b[k] -= m;
        d[k] -= m * d[k - 1];
    }
    S[n + 1] = S[n] = d[n - 1] / b[n - 1];
    for (int k = n - 2; k >= 0; k--) S[k + 1] = (d[k] - 1.0 * S[k + 2]) / b[k];
    S[0] = S[1];
    for (int i = 0; i < nd - 1; i++) {
        t.a[i] = (S[i + 1] - S[i]) / dr / dr / dr;
        t.b[i] = 3.0 * S[i] / dr / dr;
        t.c[i] = (t.d[i + 1] - t.d[i] - 2.0 * S[i] - S[i + 1]) / dr;
    }
}

double table_negligible_from(const HostTable& t, double tol) {
    const double dr = t.dr;
    int k0 = t.n - 1;  // segments [k0, n-1) are all negligible
    for (int k = t.n - 2; k >= 0; k--) {
        const double a = std::fabs(t.a[k]), b = std::fabs(t.b[k]), c = std::fabs(t.c[k]), d = std::fabs(t.d[k]);
        double vmax = d + dr * (c + dr * (b + dr * a));
        double dmax = c + dr * (2.0 * b + 3.0 * dr * a);
        if (t.rmult) {  // value / r and (slope - value / r) / r
            const double r = std::max(t.off + k * dr, 1e-12);
            dmax = (dmax + vmax / r) / r;
            vmax /= r;
        }
        if (!(vmax <= tol && dmax <= tol)) break;
        k0 = k;
    }
    return k0 >= t.n - 1 ? t.max_range() : t.off + k0 * dr;
}

bool table_read(const HostTable& t, double r, double& val, double& dval) {
    double rval = r - t.off;
    int x = (int)(rval / t.dr);
    double dx = rval - (double)x * t.dr;
    if (x > t.n - 1) {
        if (!t.allow_hi) return false;
        val = dval = t.out_hi;
        return true;
    }
    if (x < -1) {
        if (!t.allow_lo) return false;
        val = dval = t.out_lo;
        return true;
    }
    if (x == t.n - 1) {
        dx += t.dr;
        x--;
    }
    if (x == -1) x = 0;
    val = (t.d[x] + dx * (t.c[x] + dx * (t.b[x] + dx * t.a[x])));
    dval = (t.c[x] + dx * (2.0 * t.b[x] + 3.0 * dx * t.a[x]));
    if (t.rmult) {
        val /= r;
        dval = (dval - val) / r;
    }
    return true;
}

}  // namespace omdg
