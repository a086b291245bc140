// case_files.cpp -- a case from the reference's own input files, and the
// restart file rg####c.d in both directions.
//
// The Fortran host reads, in this order (A0main.f90:158-190):
//   gd####c.dat       GRID3 (Grid3.f90:31-280): extents, piecewise-linear
//                     coordinate lines, the cell map in (I4,2X,I1...) rows
//   sbc####c.dat      SETUP's &INPUT (Setup.f90:227-335), then SBC
//                     (Sbc.f90:57-355): pressure reference, inlet blocks,
//                     exhausts, wall properties, &RADIN, band edges WL
//   relaxfactorc.txt  SETUP (Setup.f90:443-509)
//   Kinetic.d         SETUP (Setup.f90:858-888)
//   it####t.dat       melt_surf_T (Initsv.f90:394-547)
//   rg####c.d         read_restart_data (Initsv.f90:225-316) when restarting
// The text files are read with the rules of Fortran list-directed input
// (values separated by blanks or commas, each READ starting on a new record
// and continuing onto the next ones while values are missing, the rest of
// the last record skipped), namelist input, and the fixed-width edit
// descriptors the reference uses.  The restart file is sequential
// unformatted with 4-byte little-endian record-length markers before and
// after each record.
#include "case_store.h"
#include "physics.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <vector>

static_assert(__BYTE_ORDER__ == __ORDER_LITTLE_ENDIAN__, "restart records are little-endian");

namespace gfm {
namespace host {
namespace {

// ---- text input ------------------------------------------------------------
struct TextFile {
    std::vector<std::string> lines;
    size_t pos = 0;
    bool load(const char* path) {
        FILE* fp = std::fopen(path, "rb");
        if (!fp) return false;
        std::string cur;
        int c;
        while ((c = std::fgetc(fp)) != EOF) {
            if (c == '\n') { lines.push_back(cur); cur.clear(); }
            else if (c != '\r') cur.push_back((char)c);
        }
        if (!cur.empty()) lines.push_back(cur);
        std::fclose(fp);
        return true;
    }
    const std::string* next() { return pos < lines.size() ? &lines[pos++] : nullptr; }
};

// list-directed value separators; a '/' ends the record's values, a '!' or
// anything after the requested count is not read
void split_values(const std::string& l, std::vector<std::string>& out, bool& slash) {
    slash = false;
    size_t i = 0;
    while (i < l.size()) {
        char c = l[i];
        if (c == ' ' || c == '\t' || c == ',') { ++i; continue; }
        if (c == '/') { slash = true; return; }
        size_t b = i;
        while (i < l.size() && l[i] != ' ' && l[i] != '\t' && l[i] != ',' && l[i] != '/') ++i;
        std::string tok = l.substr(b, i - b);
        // r*c repeat form
        size_t star = tok.find('*');
        if (star != std::string::npos && star > 0) {
            int r = std::atoi(tok.substr(0, star).c_str());
            std::string v = tok.substr(star + 1);
            for (int k = 0; k < r; ++k) out.push_back(v);
        } else {
            out.push_back(tok);
        }
    }
}

// one list-directed READ of n values
bool read_list(TextFile& f, int n, std::vector<std::string>& v) {
    v.clear();
    while ((int)v.size() < n) {
        const std::string* l = f.next();
        if (!l) return false;
        bool slash = false;
        split_values(*l, v, slash);
        if (slash) break;
    }
    if ((int)v.size() < n) return false;
    v.resize(n);
    return true;
}

bool to_double(const std::string& s, double& out) {
    std::string t(s);
    for (char& c : t)
        if (c == 'd' || c == 'D') c = 'e';
    char* end = nullptr;
    out = std::strtod(t.c_str(), &end);
    return end && end != t.c_str() && *end == '\0';
}
bool to_int(const std::string& s, int& out) {
    char* end = nullptr;
    long v = std::strtol(s.c_str(), &end, 10);
    if (!end || end == s.c_str() || *end != '\0') return false;
    out = (int)v;
    return true;
}
bool to_logical(const std::string& s, int& out) {
    std::string t;
    for (char c : s) t.push_back((char)std::toupper((unsigned char)c));
    if (!t.empty() && t[0] == '.') t = t.substr(1);
    if (t.empty()) return false;
    if (t[0] == 'T') { out = 1; return true; }
    if (t[0] == 'F') { out = 0; return true; }
    return false;
}

bool read_doubles(TextFile& f, int n, double* out) {
    std::vector<std::string> v;
    if (!read_list(f, n, v)) return false;
    for (int i = 0; i < n; ++i)
        if (!to_double(v[i], out[i])) return false;
    return true;
}
bool read_ints(TextFile& f, int n, int* out) {
    std::vector<std::string> v;
    if (!read_list(f, n, v)) return false;
    for (int i = 0; i < n; ++i) {
        double d;
        if (!to_int(v[i], out[i])) {
            if (!to_double(v[i], d)) return false;
            out[i] = (int)d;
        }
    }
    return true;
}

std::string lower(const std::string& s) {
    std::string t;
    for (char c : s) t.push_back((char)std::tolower((unsigned char)c));
    return t;
}

// namelist input: skips records up to the one that starts the group
// "&name", then collects name=value pairs up to the terminating '/'
using Namelist = std::map<std::string, std::vector<std::string>>;
bool read_namelist(TextFile& f, const char* group, Namelist& kv) {
    const std::string want = "&" + lower(group);
    std::string text;
    bool found = false;
    for (;;) {
        const std::string* l = f.next();
        if (!l) return false;
        std::string t = lower(*l);
        size_t p = t.find_first_not_of(" \t");
        if (p == std::string::npos) continue;
        if (t.compare(p, want.size(), want) == 0) {
            found = true;
            text = l->substr(p + want.size());
            break;
        }
    }
    if (!found) return false;
    // up to the '/' that ends the group (no character values are read here)
    for (;;) {
        size_t sl = text.find('/');
        if (sl != std::string::npos) { text.resize(sl); break; }
        const std::string* l = f.next();
        if (!l) return false;
        text += " " + *l;
    }
    // element designators keep their subscripts in one token: "ba_f(1,2)"
    // becomes "ba_f(1:2)"
    std::string spaced;
    int depth = 0;
    for (char c : text) {
        if (c == '(') ++depth;
        if (c == ')' && depth > 0) --depth;
        if (c == '=') spaced += " = ";
        else if (c == ',' && depth > 0) spaced.push_back(':');
        else spaced.push_back(c);
    }
    std::vector<std::string> tok;
    bool slash;
    split_values(spaced, tok, slash);
    std::string key;
    for (size_t i = 0; i < tok.size(); ++i) {
        if (i + 1 < tok.size() && tok[i + 1] == "=") { key = lower(tok[i]); kv[key]; ++i; continue; }
        if (tok[i] == "=" || key.empty()) continue;
        kv[key].push_back(tok[i]);
    }
    return true;
}
bool nl_double(const Namelist& kv, const char* k, double& v) {
    auto it = kv.find(k);
    if (it == kv.end() || it->second.empty()) return true;
    return to_double(it->second[0], v);
}
bool nl_int(const Namelist& kv, const char* k, int& v) {
    auto it = kv.find(k);
    if (it == kv.end() || it->second.empty()) return true;
    double d;
    if (to_int(it->second[0], v)) return true;
    if (!to_double(it->second[0], d)) return false;
    v = (int)d;
    return true;
}
bool nl_logical(const Namelist& kv, const char* k, int& v) {
    auto it = kv.find(k);
    if (it == kv.end() || it->second.empty()) return true;
    return to_logical(it->second[0], v);
}

// ---- gd####c.dat (Grid3.f90:31-280) -----------------------------------------
// one coordinate line: X(1..I1)=first value, then linear between listed
// points to index n-1, normalised by R0=1, X(n)=X(n-1), DX(I)=X(I+1)-X(I-1)
bool grid_line(TextFile& f, int n, std::vector<double>& x, std::vector<double>& dx) {
    x.assign(n, 0.0);
    dx.assign(n, 0.0);
    if (!f.next()) return false;   // title
    double v[2];
    if (!read_doubles(f, 2, v)) return false;
    int i1 = (int)v[0];
    if (i1 < 1 || i1 > n) return false;
    for (int i = 1; i <= i1; ++i) x[i - 1] = v[1];
    while (i1 < n - 1) {
        if (!read_doubles(f, 2, v)) return false;
        int i2 = (int)v[0];
        if (i2 <= i1) continue;   // Grid3.f90:89
        double del = (v[1] - x[i1 - 1]) / (i2 - i1);
        if (i2 > n || !(del > 0.0)) return false;   // Grid3.f90:91-97
        for (int i = i1 + 1; i <= i2; ++i) x[i - 1] = x[i - 2] + del;
        i1 = i2;
    }
    for (int i = 1; i <= n - 1; ++i) x[i - 1] = x[i - 1] / 1.0;
    x[n - 1] = x[n - 2];
    for (int i = 2; i <= n - 1; ++i) dx[i - 1] = x[i] - x[i - 2];
    return true;
}

int read_gd(const char* path, CaseStore& s, int& nr0) {
    TextFile f;
    if (!f.load(path)) return GFM_E_IO;
    if (!f.next() || !f.next()) return GFM_E_IO;   // two titles
    double h[10];
    if (!read_doubles(f, 10, h)) return GFM_E_IO;
    const int mp = (int)h[1], np = (int)h[2], lp = (int)h[3];
    const int ndp0 = (int)h[6], npt0 = (int)h[7];
    nr0 = (int)h[9];
    // cartesian grids of at least 6 positions per direction (the NP<6 and
    // LP<6 branches of Grid3.f90:155-164, 204-211 are 2-D cases)
    if (mp < 6 || np < 6 || lp < 6 || (mp & 1) || (np & 1) || (lp & 1) || mp > 8192 || np > 8192 || lp > 8192)
        return GFM_E_UNSUPPORTED;
    if (ndp0 + npt0 != 0) return GFM_E_UNSUPPORTED;   // droplet / particle phases
    if (nr0 < 1 || nr0 > 100000) return GFM_E_IO;
    s.mp = mp; s.np = np; s.lp = lp;
    if (!grid_line(f, mp, s.x, s.dx)) return GFM_E_IO;
    if (!grid_line(f, np, s.r, s.dr)) return GFM_E_IO;
    if (!grid_line(f, lp, s.z, s.dz)) return GFM_E_IO;
    s.rs.assign(np, 1.0);
    // cell map: layers up to K2, rows up to I2, one digit per even J
    s.ibcell.assign(s.n(), 0);
    if (!f.next()) return GFM_E_IO;   // title
    int k1 = 0;
    while (k1 < lp) {
        int k2;
        if (!read_ints(f, 1, &k2)) return GFM_E_IO;
        if (k2 <= k1 || k2 > lp) return GFM_E_IO;
        int i1 = 0;
        while (i1 < mp) {
            const std::string* l = f.next();
            if (!l) return GFM_E_IO;
            // (I4,2X,<NP>I1): columns 1-4, then one column per J=2,4,..,NP;
            // blank columns read as 0
            std::string c4 = l->substr(0, l->size() < 4 ? l->size() : 4);
            int i2 = 0;
            bool any = false;
            for (char c : c4) {
                if (c == ' ') continue;
                if (c < '0' || c > '9') return GFM_E_IO;
                i2 = i2 * 10 + (c - '0');
                any = true;
            }
            if (!any || i2 <= i1 || i2 > mp) return GFM_E_IO;
            std::vector<int> ibc(np + 1, 0);
            for (int j = 2; j <= np; j += 2) {
                size_t col = 6 + (size_t)(j / 2 - 1);
                char c = col < l->size() ? (*l)[col] : ' ';
                int d = 0;
                if (c != ' ') {
                    if (c < '0' || c > '9') return GFM_E_IO;
                    d = c - '0';
                }
                if (d > 5) d -= 10;   // Grid3.f90:242
                // half-blocked cells: -1 and -2 index BV_F(2) and BA_F(3,2)
                // (Grid3.f90:12); digits 6 and 7 would index past them
                if (d < -2) return GFM_E_UNSUPPORTED;
                ibc[j] = d;
            }
            for (int k = k1 + 2; k <= k2; k += 2)
                for (int i = i1 + 2; i <= i2; i += 2)
                    for (int j = 2; j <= np; j += 2) s.ibcell[s.at(i, j, k)] = (int16_t)ibc[j];
            i1 = i2;
        }
        k1 = k2;
    }
    // &GRD: the half-block factors (Grid3.f90:252-255); absent, they stay 1
    Namelist kv;
    if (read_namelist(f, "GRD", kv)) {
        for (const auto& it : kv) {
            const std::string& key = it.first;
            const size_t par = key.find('(');
            const std::string name = key.substr(0, par);
            int dims[2];
            double* dst;
            double bd[6];
            if (name == "bv_f") { dims[0] = 2; dims[1] = 1; dst = s.bv_f; }
            else if (name == "ba_f") { dims[0] = 3; dims[1] = 2; dst = s.ba_f; }
            else if (name == "bd_f") { dims[0] = 3; dims[1] = 2; dst = bd; }   // declared, used nowhere
            else return GFM_E_IO;
            // first element: the subscripts of an element designator, else (1,1)
            int sub[2] = {1, 1};
            if (par != std::string::npos) {
                const size_t end = key.find(')', par);
                if (end == std::string::npos) return GFM_E_IO;
                std::string inner = key.substr(par + 1, end - par - 1);
                int ns = 0;
                size_t b = 0;
                while (b <= inner.size() && ns < 2) {
                    size_t e = inner.find(':', b);
                    if (e == std::string::npos) e = inner.size();
                    int v;
                    if (!to_int(inner.substr(b, e - b), v)) return GFM_E_IO;
                    sub[ns++] = v;
                    b = e + 1;
                }
                if (sub[0] < 1 || sub[0] > dims[0] || sub[1] < 1 || sub[1] > dims[1]) return GFM_E_IO;
            }
            int pos = (sub[0] - 1) + dims[0] * (sub[1] - 1);   // column-major, as Fortran stores them
            for (const std::string& v : it.second) {
                if (pos >= dims[0] * dims[1]) return GFM_E_IO;
                double x;
                if (!to_double(v, x)) return GFM_E_IO;
                dst[pos++] = x;
            }
        }
        for (int q = 0; q < 8; ++q) {
            const double v = q < 2 ? s.bv_f[q] : s.ba_f[q - 2];
            if (!(v > 0.0 && v < 1.0e30)) return GFM_E_IO;
        }
    }
    return GFM_OK;
}

// ---- sbc####c.dat ---------------------------------------------------------------
struct SbcExtra {
    int irstyp = 0, id_rad = 0, n_exh = 0, n_wall = 0, nwl = 1;
};

int read_sbc(const char* path, CaseInputs& in, SbcExtra& ex) {
    TextFile f;
    if (!f.load(path)) return GFM_E_IO;
    Namelist kv;
    if (!read_namelist(f, "INPUT", kv)) return GFM_E_IO;
    bool ok = nl_double(kv, "gmfr", in.gmfr) && nl_double(kv, "pg0", in.pg0) && nl_double(kv, "q0", in.q0_jkg) &&
              nl_double(kv, "t_init", in.t_init_k) && nl_double(kv, "bgcon", in.bgcon) &&
              nl_double(kv, "gmu_ref", in.gmu_ref) && nl_int(kv, "maxgi", in.maxgi) &&
              nl_logical(kv, "react", in.react) && nl_int(kv, "irstyp", ex.irstyp) &&
              nl_int(kv, "id_rad", ex.id_rad) && nl_int(kv, "interval_rad", in.interval_rad) &&
              nl_int(kv, "initial_gitr", in.initial_gitr) && nl_int(kv, "ms", in.ms) &&
              nl_int(kv, "irstypm", in.irstypm) && nl_int(kv, "maxms", in.maxms) && nl_double(kv, "bmcon", in.bmcon) &&
              nl_double(kv, "aform", in.aform) && nl_double(kv, "aoxid", in.aoxid) && nl_double(kv, "esf", in.esf) &&
              nl_double(kv, "eso", in.eso);
    if (!ok) return GFM_E_IO;
    // pressure reference (Sbc.f90:57)
    {
        std::vector<std::string> v;
        if (!read_list(f, 4, v)) return GFM_E_IO;
        double pr;
        if (!to_int(v[0], in.i_ref) || !to_int(v[1], in.j_ref) || !to_int(v[2], in.k_ref) || !to_double(v[3], pr))
            return GFM_E_IO;
        in.p_ref_pa = pr;
    }
    // inlet blocks up to a row of zeros (Sbc.f90:66-76)
    for (;;) {
        int b7[7];
        if (!read_ints(f, 7, b7)) return GFM_E_IO;
        if (b7[0] <= 0) break;
        double st[10];
        if (!read_doubles(f, 10, st)) return GFM_E_IO;
        InletBlock b;
        b.i1 = b7[0]; b.j1 = b7[1]; b.k1 = b7[2]; b.i2 = b7[3]; b.j2 = b7[4]; b.k2 = b7[5]; b.iu = b7[6];
        b.t_k = st[0]; b.yf = st[1]; b.yox = st[2]; b.yn2 = st[3]; b.yco2 = st[4]; b.yh2o = st[5]; b.yck = st[6];
        b.u = st[7]; b.v = st[8]; b.w = st[9];
        in.inlets.push_back(b);
    }
    // exhausts (Sbc.f90:273-284): box, then orientation, direction, type
    // (0: a fraction of the mean wall T, else fixed), fraction, fixed T
    if (!f.next()) return GFM_E_IO;   // "Exhausts:"
    if (!read_ints(f, 1, &ex.n_exh) || ex.n_exh < 0 || ex.n_exh > 100000) return GFM_E_IO;
    if (ex.n_exh > GFM_MAX_EXHAUSTS) return GFM_E_UNSUPPORTED;
    in.wall.nex = ex.n_exh;
    for (int n = 0; n < ex.n_exh; ++n) {
        int e6[6];
        if (!read_ints(f, 6, e6)) return GFM_E_IO;
        std::vector<std::string> v;
        if (!read_list(f, 5, v)) return GFM_E_IO;
        gfm_wall_spec& w = in.wall;
        w.exh_i1[n] = e6[0]; w.exh_j1[n] = e6[1]; w.exh_k1[n] = e6[2];
        w.exh_i2[n] = e6[3]; w.exh_j2[n] = e6[4]; w.exh_k2[n] = e6[5];
        if (!to_int(v[0], w.exh_orient[n]) || !to_int(v[1], w.exh_direct[n]) || !to_int(v[2], w.exh_type[n]) ||
            !to_double(v[3], w.exh_frac[n]) || !to_double(v[4], w.exh_fixed[n]))
            return GFM_E_IO;
    }
    // wall properties up to a row of zeros (Sbc.f90:290-313)
    if (!f.next()) return GFM_E_IO;   // "Wall Properties:"
    for (int n = 0; n < 1000; ++n) {
        int w7[7];
        if (!read_ints(f, 7, w7)) return GFM_E_IO;
        if (w7[0] <= 0) break;
        double w4[4];
        if (!read_doubles(f, 4, w4)) return GFM_E_IO;
        ++ex.n_wall;
    }
    // &RADIN with the defaults of Sbc.f90:319-334, then the band edges in um
    Namelist rk;
    if (!read_namelist(f, "RADIN", rk)) return GFM_E_IO;
    ex.nwl = 1;
    in.ri = 1.0; in.h_g = 10.0;
    if (!nl_int(rk, "nwl", ex.nwl) || !nl_double(rk, "ri", in.ri) || !nl_double(rk, "h_g", in.h_g)) return GFM_E_IO;
    {
        gfm_wall_spec& w = in.wall;
        if (!nl_double(rk, "t_a", w.t_a) || !nl_double(rk, "h_a", w.h_a) || !nl_double(rk, "w_k", w.w_k) ||
            !nl_double(rk, "w_d", w.w_d) || !nl_double(rk, "eps_w", w.eps_w) || !nl_double(rk, "eps_m", w.eps_m) ||
            !nl_double(rk, "eps_c", w.eps_c) || !nl_int(rk, "have_crown", w.have_crown) ||
            !nl_double(rk, "height_to_ceiling", w.height_to_ceiling) || !nl_int(rk, "maxri1", w.maxri1) ||
            !nl_int(rk, "maxri2", w.maxri2) || !nl_int(rk, "minri2", w.minri2))
            return GFM_E_IO;
    }
    if (ex.nwl < 1 || ex.nwl > 16) return GFM_E_UNSUPPORTED;
    in.wl_m.resize(ex.nwl);
    if (!read_doubles(f, ex.nwl, in.wl_m.data())) return GFM_E_IO;
    for (double& w : in.wl_m) w = w * 1.0e-6;
    return GFM_OK;
}

// ---- relaxfactorc.txt (Setup.f90:443-509) -------------------------------------
int read_relax(const char* path, CaseInputs& in) {
    TextFile f;
    if (!f.load(path)) return GFM_E_IO;
    double v;
    auto one = [&](double& dst) { return read_doubles(f, 1, &dst); };
    if (!f.next()) return GFM_E_IO;
    if (!one(v)) return GFM_E_IO;
    for (double& r : in.rfl) r = v;
    for (int l = 0; l < 7; ++l)
        if (!one(in.rfl[l])) return GFM_E_IO;
    if (!f.next()) return GFM_E_IO;
    if (!one(v)) return GFM_E_IO;
    for (double& r : in.rf) r = v;
    if (!one(in.rf[0]) || !one(in.rf[1]) || !one(in.rf[2]) || !one(in.rf[17]) || !one(in.rf[20])) return GFM_E_IO;
    if (!one(in.rf_tsurf)) return GFM_E_IO;
    if (!one(in.rfm) || !one(in.rfm_soot)) return GFM_E_IO;   // minor species and soot
    if (!f.next()) return GFM_E_IO;
    if (!one(in.rf_hsource) || !one(in.rf_soot_form) || !one(in.rf_soot_oxid)) return GFM_E_IO;
    if (!one(v) || !one(v)) return GFM_E_IO;   // soot calibration (rf_aform, rf_afover)
    if (!one(in.soot_cap) || !one(in.t0_sf) || !one(in.t0_so)) return GFM_E_IO;
    if (!f.next()) return GFM_E_IO;
    int g;
    if (!read_ints(f, 1, &g)) return GFM_E_IO;
    for (int& n : in.ntimesg) n = g;
    for (int n = 0; n < 12; ++n)
        if (!read_ints(f, 1, &in.ntimesg[n])) return GFM_E_IO;
    if (!read_ints(f, 1, &in.ntimesm)) return GFM_E_IO;   // minor species (Setup.f90:510-511)
    return GFM_OK;
}

// ---- it####t.dat (Initsv.f90:423-455) -------------------------------------------
double fixed_field(const std::string& l, size_t b, size_t w, bool& ok) {
    if (b >= l.size()) return 0.0;   // padded with blanks
    std::string t = l.substr(b, w);
    size_t p = t.find_first_not_of(' ');
    if (p == std::string::npos) return 0.0;
    size_t e = t.find_last_not_of(' ');
    double v;
    if (!to_double(t.substr(p, e - p + 1), v)) ok = false;
    return v;
}

int read_it(const char* path, int mz, int nz, CaseInputs& in) {
    TextFile f;
    if (!f.load(path)) return GFM_E_IO;
    int itn;
    double q_melt_req, qls, surf;
    if (!read_ints(f, 1, &itn) || !read_doubles(f, 1, &q_melt_req) || !read_doubles(f, 1, &qls) ||
        !read_doubles(f, 1, &surf))
        return GFM_E_IO;
    in.have_it = true;
    in.itn = itn;
    in.surf_t = surf;
    in.tgs.assign((size_t)mz * nz, surf);
    if (itn > 0) {
        if (!f.next() || !f.next()) return GFM_E_IO;
        int jb = 1;
        for (;;) {
            int je = jb + 10;
            if (je > nz) je = nz;
            if (!f.next() || !f.next()) return GFM_E_IO;
            for (int i = 1; i <= mz; ++i) {   // (F11.3,11F11.1)
                const std::string* l = f.next();
                if (!l) return GFM_E_IO;
                bool ok = true;
                for (int j = jb; j <= je; ++j)
                    in.tgs[(i - 1) + (size_t)mz * (j - 1)] = fixed_field(*l, 11 + 11 * (size_t)(j - jb), 11, ok);
                if (!ok) return GFM_E_IO;
            }
            jb = je + 1;
            if (jb > nz) break;
        }
    }
    return GFM_OK;
}

// ---- sequential unformatted records ------------------------------------------------
struct RecReader {
    FILE* fp = nullptr;
    // reads one record of exactly `bytes` payload bytes
    bool rec(void* dst, size_t bytes) {
        uint32_t a, b;
        if (std::fread(&a, 4, 1, fp) != 1 || a != bytes) return false;
        if (bytes && std::fread(dst, 1, bytes, fp) != bytes) return false;
        if (std::fread(&b, 4, 1, fp) != 1 || b != a) return false;
        return true;
    }
};
struct RecWriter {
    FILE* fp = nullptr;
    bool rec(const void* src, size_t bytes) {
        uint32_t a = (uint32_t)bytes;
        return std::fwrite(&a, 4, 1, fp) == 1 && (bytes == 0 || std::fwrite(src, 1, bytes, fp) == bytes) &&
               std::fwrite(&a, 4, 1, fp) == 1;
    }
};

constexpr int kLend = 7;   // GF(1:LEND) in the restart file (Var_mod.f90:125)

}  // namespace

int read_restart(const char* path, CaseStore& s, const gfm_params& P, gfm_fields& F, gfm_restart_tail& tail,
                 int& maxgi) {
    const int mp = s.mp, np = s.np, lp = s.lp;
    const long N = s.n();
    RecReader r;
    r.fp = std::fopen(path, "rb");
    if (!r.fp) return GFM_E_IO;
    auto IB = [&](int i, int j, int k) { return (int)s.ibcell[s.at(i, j, k)]; };
    const int itr_gas0 = 0;   // a real restart, not a loop-forced one
    for (int i = 2; i <= mp; i += 2)
        for (int j = 2; j <= np; j += 2)
            for (int k = 2; k <= lp; k += 2) {
                double g[6], gff[kLend];
                if (!r.rec(g, sizeof g) || !r.rec(gff, sizeof gff)) { std::fclose(r.fp); return GFM_E_IO; }
                const long a = s.at(i, j, k);
                s.p[a] = g[0];
                if (IB(i, j, k) == 2 && itr_gas0 <= 0) {
                    s.gf[a + gfm::kK * N] = gff[gfm::kK];
                    s.gf[a + gfm::kEps * N] = gff[gfm::kEps];
                    continue;
                }
                if (i < mp && IB(i + 1, j, k) != 2 && IB(i + 1, j, k) != 1) s.ug[s.at(i + 1, j, k)] = g[1];
                if (j < np && IB(i, j + 1, k) != 2 && IB(i, j + 1, k) != 1) s.ug[s.at(i, j + 1, k) + N] = g[2];
                if (k < lp && IB(i, j, k + 1) != 2 && IB(i, j, k + 1) != 1) s.ug[s.at(i, j, k + 1) + 2 * N] = g[3];
                if (IB(i, j, k) != 4) s.t[a] = g[4];   // the melt surface keeps melt_surf_T's value
                s.theta[a] = g[5];
                for (int l = 0; l < kLend; ++l) s.gf[a + (long)l * N] = gff[l];
                prop_dnst(s, P, a);
                prop_ther(s, P, a);
            }
    const int mz = mp / 2, nz = np / 2;
    s.t_surf_prev.assign((size_t)mz * nz, 0.0);
    double ff[2];
    int32_t q1 = 0, rd = 0;
    if (!r.rec(s.bs_hprev.data(), sizeof(double) * N) ||
        !r.rec(s.t_surf_prev.data(), sizeof(double) * s.t_surf_prev.size()) || !r.rec(ff, sizeof ff) ||
        !r.rec(&q1, 4) || !r.rec(&rd, 4)) {
        std::fclose(r.fp);
        return GFM_E_IO;
    }
    F.factor = ff[0];
    F.fadj = ff[1];
    F.i1st_rad_qe_done = q1;
    tail.i1st_rad_done = rd == 1 ? 1 : 0;
    // the last three records may be absent in older files (Initsv.f90:296-303)
    int32_t itr = 0, ir2[2] = {0, 0}, ivr = 0;
    if (r.rec(&itr, 4)) {
        F.itr_gas = itr;
        if (r.rec(ir2, 8)) {
            tail.itr_rad = ir2[0];
            tail.itr_gend = ir2[1];
            if (r.rec(&ivr, 4) && (tail.itr_gend <= F.itr_gas || ivr != tail.interval_rad))
                tail.itr_gend = F.itr_gas + tail.interval_rad;
        }
    }
    std::fclose(r.fp);
    maxgi = maxgi + itr;
    return GFM_OK;
}

// The radiation restart's first four records: QE, QA, QL (MZ,NZ,LZ) and
// wall_rad_T (MP,NP,LP), K slowest; the rest (the RAD0/QRNF totals and the
// boundary patches' state) belongs to the wall exchange and is restored on a
// handle (gfm_gpu_wall_put).  A wall cell centre with wall_rad_T > 0 takes
// that temperature and its enthalpy (Rad_emis.f90:91-100).
int read_rad_restart(const char* path, CaseStore& s, const gfm_params& P) {
    const int mp = s.mp, np = s.np, lp = s.lp;
    const size_t ncell = (size_t)(mp / 2) * (np / 2) * (lp / 2), N = (size_t)s.n();
    std::vector<double> ql(ncell), wt(N);
    RecReader r;
    r.fp = std::fopen(path, "rb");
    if (!r.fp) return GFM_E_IO;
    s.qe.assign(ncell, 0.0);
    s.qa.assign(ncell, 0.0);
    const bool ok = r.rec(s.qe.data(), ncell * sizeof(double)) && r.rec(s.qa.data(), ncell * sizeof(double)) &&
                    r.rec(ql.data(), ncell * sizeof(double)) && r.rec(wt.data(), N * sizeof(double));
    std::fclose(r.fp);
    if (!ok) return GFM_E_IO;
    for (int k = lp; k >= 2; k -= 2)
        for (int i = 2; i <= mp; i += 2)
            for (int j = 2; j <= np; j += 2) {
                const long a = s.at(i, j, k);
                if (wt[a] > 0.0) {
                    s.t[a] = wt[a] / P.t0;
                    prop_t2h(s, P, a);
                }
            }
    return GFM_OK;
}

}  // namespace host
}  // namespace gfm

using gfm::host::CaseInputs;
using gfm::host::CaseStore;

extern "C" int gfm_case_read(const gfm_case_files* files, const gfm_case_options* opt, gfm_case* out,
                             gfm_case_summary* summary) {
    if (!files || !out || !files->gd || !files->sbc || !files->relax || !files->kinetic) return GFM_E_ARG;
    std::memset(out, 0, sizeof *out);
    if (summary) std::memset(summary, 0, sizeof *summary);
    CaseStore* S = new (std::nothrow) CaseStore;
    if (!S) return GFM_E_NOMEM;
    CaseInputs in;
    gfm::host::SbcExtra ex;
    int rc = gfm::host::read_gd(files->gd, *S, in.nr0);
    if (rc == GFM_OK) rc = gfm::host::read_sbc(files->sbc, in, ex);
    if (rc == GFM_OK) rc = gfm::host::read_relax(files->relax, in);
    if (rc == GFM_OK && files->it) rc = gfm::host::read_it(files->it, S->mp / 2, S->np / 2, in);
    if (rc != GFM_OK) { delete S; return rc; }
    const double sig0[12] = {0.7, 0.7, 0.7, 1.0, 1.0, 0.7, 0.7, 0.7, 0.7, 0.7, 0.7, 0.7};   // Var_mod.f90:211-212
    for (int i = 0; i < 12; ++i) in.sigma[i] = sig0[i];
    in.kappa.assign(ex.nwl, 0.0);
    if (opt) {
        if (opt->sigma_eps > 0) in.sigma[4] = opt->sigma_eps;
        in.wall_sink = opt->wall_sink;
        if (opt->t_wall_k > 0) in.t_wall_k = opt->t_wall_k;
        in.rad_emission = opt->rad_emission;
        for (int l = 0; l < ex.nwl; ++l) in.kappa[l] = opt->kappa[l];
        if (opt->maxgi > 0) in.maxgi = opt->maxgi;
        in.adi_mode = opt->adi_mode;
        in.precision = opt->precision;
        if (opt->gas_model && !in.ms) { delete S; return GFM_E_ARG; }
        in.gas_model = opt->gas_model;
    }
    in.rg_path = files->rg;
    in.rr_path = files->rr;
    rc = gfm::host::finish_case(S, in, files->kinetic, out, summary);
    if (rc != GFM_OK) return rc;
    if (summary) {
        summary->irstyp = ex.irstyp;
        summary->id_rad = ex.id_rad;
        summary->n_exhausts = ex.n_exh;
        summary->n_wall_blocks = ex.n_wall;
    }
    return GFM_OK;
}

extern "C" int gfm_restart_write(const char* path, const gfm_grid* grid, const gfm_fields* f,
                                 const gfm_restart_tail* tail) {
    if (!path || !grid || !f || !tail || !f->p || !f->ug || !f->t || !f->theta || !f->gf || !f->bs_hprev)
        return GFM_E_ARG;
    const int mp = grid->mp, np = grid->np, lp = grid->lp;
    if (mp < 4 || np < 4 || lp < 4 || tail->mz != mp / 2 || tail->nz != np / 2 || !tail->t_surf_prev) return GFM_E_ARG;
    const long N = (long)mp * np * lp;
    auto at = [&](int i, int j, int k) { return (i - 1) + (long)mp * ((j - 1) + (long)np * (k - 1)); };
    gfm::host::RecWriter w;
    w.fp = std::fopen(path, "wb");
    if (!w.fp) return GFM_E_IO;
    bool ok = true;
    for (int i = 2; i <= mp && ok; i += 2)
        for (int j = 2; j <= np && ok; j += 2)
            for (int k = 2; k <= lp && ok; k += 2) {
                const long a = at(i, j, k);
                double g[6];
                g[0] = f->p[a];
                g[1] = f->ug[i == mp ? at(mp - 1, j, k) : at(i + 1, j, k)];
                g[2] = f->ug[(j == np ? at(i, np - 1, k) : at(i, j + 1, k)) + N];
                g[3] = f->ug[(k == lp ? at(i, j, lp - 1) : at(i, j, k + 1)) + 2 * N];
                g[4] = f->t[a];
                g[5] = f->theta[a];
                double gff[gfm::host::kLend];
                for (int l = 0; l < gfm::host::kLend; ++l) gff[l] = f->gf[a + (long)l * N];
                ok = w.rec(g, sizeof g) && w.rec(gff, sizeof gff);
            }
    const double ff[2] = {f->factor, f->fadj};
    const int32_t q1 = f->i1st_rad_qe_done, rd = tail->i1st_rad_done, itr = f->itr_gas;
    const int32_t ir2[2] = {tail->itr_rad, tail->itr_gend}, ivr = tail->interval_rad;
    ok = ok && w.rec(f->bs_hprev, sizeof(double) * N) &&
         w.rec(tail->t_surf_prev, sizeof(double) * (size_t)tail->mz * tail->nz) && w.rec(ff, sizeof ff) &&
         w.rec(&q1, 4) && w.rec(&rd, 4) && w.rec(&itr, 4) && w.rec(ir2, 8) && w.rec(&ivr, 4);
    if (std::fclose(w.fp) != 0) ok = false;
    return ok ? GFM_OK : GFM_E_IO;
}

// ---- the minor species restart rs####c.d (Sav3f.f90:96-117, Initsv.f90:350-372) ----
namespace {
bool minor_arrays(const gfm_minor* m) {
    return m && m->gfm && m->smf && m->bs_soot_prev && m->sfp_soot_prev && m->rrms;
}
}  // namespace

extern "C" int gfm_minor_read(const char* path, const gfm_grid* grid, gfm_minor* out) {
    if (!path || !grid || !minor_arrays(out)) return GFM_E_ARG;
    const int mp = grid->mp, np = grid->np, lp = grid->lp;
    if (mp < 4 || np < 4 || lp < 4) return GFM_E_ARG;
    const long N = (long)mp * np * lp, NCA = (long)(mp / 2) * (np / 2) * (lp / 2);
    auto at = [&](int i, int j, int k) { return (i - 1) + (long)mp * ((j - 1) + (long)np * (k - 1)); };
    gfm::host::RecReader r;
    r.fp = std::fopen(path, "rb");
    if (!r.fp) return GFM_E_IO;
    bool ok = true;
    for (int i = 2; i <= mp && ok; i += 2)
        for (int j = 2; j <= np && ok; j += 2)
            for (int k = 2; k <= lp && ok; k += 2) {
                double g[GFM_NSP_MINOR + 1];
                ok = r.rec(g, sizeof g);
                if (!ok) break;
                const long a = at(i, j, k);
                for (int l = 0; l < GFM_NSP_MINOR; ++l) out->gfm[a + (long)l * N] = g[l];
                out->smf[a] = g[GFM_NSP_MINOR];
            }
    int32_t itr = 0;
    ok = ok && r.rec(out->bs_soot_prev, sizeof(double) * N) && r.rec(out->sfp_soot_prev, sizeof(double) * N) &&
         r.rec(out->rrms, sizeof(double) * 5 * NCA) && r.rec(&itr, 4);
    std::fclose(r.fp);
    if (!ok) return GFM_E_IO;
    out->itr_ms = itr;
    out->imscon = 0;
    return GFM_OK;
}

extern "C" int gfm_minor_write(const char* path, const gfm_grid* grid, const gfm_minor* m) {
    if (!path || !grid || !minor_arrays(m)) return GFM_E_ARG;
    const int mp = grid->mp, np = grid->np, lp = grid->lp;
    if (mp < 4 || np < 4 || lp < 4) return GFM_E_ARG;
    const long N = (long)mp * np * lp, NCA = (long)(mp / 2) * (np / 2) * (lp / 2);
    auto at = [&](int i, int j, int k) { return (i - 1) + (long)mp * ((j - 1) + (long)np * (k - 1)); };
    gfm::host::RecWriter w;
    w.fp = std::fopen(path, "wb");
    if (!w.fp) return GFM_E_IO;
    bool ok = true;
    for (int i = 2; i <= mp && ok; i += 2)
        for (int j = 2; j <= np && ok; j += 2)
            for (int k = 2; k <= lp && ok; k += 2) {
                const long a = at(i, j, k);
                double g[GFM_NSP_MINOR + 1];
                for (int l = 0; l < GFM_NSP_MINOR; ++l) g[l] = m->gfm[a + (long)l * N];
                g[GFM_NSP_MINOR] = m->smf[a];
                ok = w.rec(g, sizeof g);
            }
    const int32_t itr = m->itr_ms;
    ok = ok && w.rec(m->bs_soot_prev, sizeof(double) * N) && w.rec(m->sfp_soot_prev, sizeof(double) * N) &&
         w.rec(m->rrms, sizeof(double) * 5 * NCA) && w.rec(&itr, 4);
    if (std::fclose(w.fp) != 0) ok = false;
    return ok ? GFM_OK : GFM_E_IO;
}

// ---- the synthetic furnace as a case directory ----------------------------------
namespace {

struct Out {
    FILE* fp = nullptr;
    bool ok = true;
    explicit Out(const std::string& path) : fp(std::fopen(path.c_str(), "wb")) { ok = fp != nullptr; }
    ~Out() { if (fp) std::fclose(fp); }
    // CR-LF line ends, as the reference's case files have them
    void line(const std::string& s) {
        if (ok && (std::fwrite(s.data(), 1, s.size(), fp) != s.size() || std::fwrite("\r\n", 1, 2, fp) != 2)) ok = false;
    }
    bool close() {
        bool r = ok && std::fclose(fp) == 0;
        fp = nullptr;
        return r;
    }
};

// shortest decimal that reads back as the same double
std::string num(double v) {
    char b[40];
    for (int p = 15; p <= 17; ++p) {
        std::snprintf(b, sizeof b, "%.*g", p, v);
        if (std::strtod(b, nullptr) == v) break;
    }
    std::string s(b);
    if (s.find_first_of(".eEn") == std::string::npos) s += ".";   // a real, as the GUI writes them
    return s;
}

}  // namespace

extern "C" int gfm_case_write_files(const gfm_case_spec* sp, const char* dir, const char* runum) {
    using namespace gfm::host;
    if (!sp || !dir || !runum || std::strlen(runum) == 0 || std::strlen(runum) > 16) return GFM_E_ARG;
    // what the files cannot carry: the seeded perturbation of the fresh
    // start and a turbulent Prandtl number of k other than the reference's
    if (sp->noise_amp != 0.0 || sp->sigma_k != 1.0) return GFM_E_UNSUPPORTED;
    CaseStore s;
    CaseInputs in;
    int rc = synth_inputs(sp, s, in);
    if (rc != GFM_OK) return rc;
    const std::string d(dir), r(runum);
    const int mp = s.mp, np = s.np, lp = s.lp;
    auto IB = [&](int i, int j, int k) { return (int)s.ibcell[s.at(i, j, k)]; };

    {   // gd####c.dat: coordinate lines by their two ends, cell map by runs
        Out f(d + "/gd" + r + "c.dat");
        f.line("Combustion Space");
        f.line("    r0, mp, np, lp, surf_length_c, surf_width_c, ndp0, npt0, nsp0, nr0, grid_type");
        f.line("    1.0 " + std::to_string(mp) + " " + std::to_string(np) + " " + std::to_string(lp) + " 0 0 0 0 7 " +
               std::to_string(in.nr0) + " 1");
        const char* titles[3] = {"X grid points", "Y grid points", "Z grid points"};
        const int ext[3] = {mp, np, lp};
        const double len[3] = {sp->lx, sp->ly, sp->lz};
        for (int a = 0; a < 3; ++a) {
            f.line(titles[a]);
            f.line("   3   0.");
            f.line("  " + std::to_string(ext[a] - 1) + "   " + num(len[a]));
        }
        f.line("Computational and blocked cells");
        auto row = [&](int i, int k) {
            std::string t;
            for (int j = 2; j <= np; j += 2) {
                const int v = IB(i, j, k);
                t.push_back((char)('0' + (v < 0 ? v + 10 : v)));   // half-blocked -1, -2 as 9, 8
            }
            return t;
        };
        auto layer = [&](int k) {
            std::vector<std::string> v;
            for (int i = 2; i <= mp; i += 2) v.push_back(row(i, k));
            return v;
        };
        for (int k = 2; k <= lp; k += 2) {
            std::vector<std::string> cur = layer(k);
            if (k < lp && layer(k + 2) == cur) continue;   // the layer holds up to the next listed K
            char b[16];
            std::snprintf(b, sizeof b, "%4d", k);
            f.line(b);
            for (int n = 0; n < (int)cur.size(); ++n) {
                if (n + 1 < (int)cur.size() && cur[n + 1] == cur[n]) continue;
                std::snprintf(b, sizeof b, "%4d  ", 2 * n + 2);
                f.line(b + cur[n]);
            }
        }
        f.line("");
        f.line("&GRD");
        f.line("/");
        if (!f.close()) return GFM_E_IO;
    }
    {   // sbc####c.dat
        Out f(d + "/sbc" + r + "c.dat");
        f.line("&INPUT");
        f.line(std::string("   REACT=") + (in.react ? ".TRUE." : ".FALSE."));
        f.line("   IRSTYP=0,MAXGI=" + std::to_string(in.maxgi) + ",ID_RAD=" + (sp->rad_emission ? "1" : "-1"));
        f.line("   MS=0,interval_rad=" + std::to_string(in.interval_rad));
        f.line("   GMFR=" + num(in.gmfr));
        f.line("   PG0=" + num(in.pg0));
        f.line("   Q0=" + num(in.q0_jkg));
        f.line("   BGCON=" + num(in.bgcon));
        f.line("   T_init=" + num(in.t_init_k));
        f.line("   initial_gitr=" + std::to_string(in.initial_gitr));
        f.line("/");
        f.line(" " + std::to_string(in.i_ref) + " " + std::to_string(in.j_ref) + " " + std::to_string(in.k_ref) + " " +
               num(in.p_ref_pa));
        for (const InletBlock& b : in.inlets) {
            f.line(" " + std::to_string(b.i1) + " " + std::to_string(b.j1) + " " + std::to_string(b.k1) + " " +
                   std::to_string(b.i2) + " " + std::to_string(b.j2) + " " + std::to_string(b.k2) + " " +
                   std::to_string(b.iu));
            f.line(" " + num(b.t_k) + " " + num(b.yf) + " " + num(b.yox) + " " + num(b.yn2) + " " + num(b.yco2) + " " +
                   num(b.yh2o) + " " + num(b.yck) + " " + num(b.u) + " " + num(b.v) + " " + num(b.w));
        }
        f.line(" 0 0 0 0 0 0 0");
        f.line("Exhausts:");
        // the flue: exit cells on the x=lx wall, x-normal, positive direction,
        // fixed radiation temperature
        int j1 = np, j2 = 0, k1 = lp, k2 = 0;
        for (int k = 2; k <= lp; k += 2)
            for (int j = 2; j <= np; j += 2)
                if (IB(mp, j, k) == 3) { j1 = std::min(j1, j); j2 = std::max(j2, j); k1 = std::min(k1, k); k2 = std::max(k2, k); }
        f.line(" 1");
        f.line(" " + std::to_string(mp) + " " + std::to_string(j1) + " " + std::to_string(k1) + " " + std::to_string(mp) +
               " " + std::to_string(j2) + " " + std::to_string(k2));
        f.line(" 1 0 1 0.9 " + num(sp->t_wall_k));
        f.line("Wall Properties:");
        f.line(" 0 0 0 0 0 0 0");
        f.line("&RADIN");
        f.line("   NWL=" + std::to_string(sp->nwl) + ",RI=" + num(in.ri) + ",H_G=" + num(in.h_g));
        f.line("/");
        std::string wl;
        for (int l = 0; l < sp->nwl; ++l) wl += (l ? " " : "") + num(sp->wl_um[l]);
        f.line(wl);
        if (!f.close()) return GFM_E_IO;
    }
    {   // relaxfactorc.txt, in the reference's line order (Setup.f90:443-509)
        Out f(d + "/relaxfactorc.txt");
        f.line("!Relaxation factors for equation loops");
        f.line(num(0.6) + " ! general value");
        for (int l = 0; l < 7; ++l) f.line(num(in.rfl[l]));
        f.line("!Relaxation factors for certain variables");
        f.line(num(0.7) + " ! general value");
        for (int l : {0, 1, 2, 17, 20}) f.line(num(in.rf[l]));
        f.line(num(in.rf_tsurf) + " ! surface temperature");
        f.line("0.5 ! minor species");
        f.line("0.2 ! soot");
        f.line("!Soot related relaxation factors and bounds");
        f.line(num(in.rf_hsource) + " ! enthalpy source term");
        for (const char* v : {"0.3", "0.3", "0.3", "0.8", "4.0d-3", "0.0", "0.0"}) f.line(v);
        f.line("!Number of sweeps in equation solver for specified items");
        f.line("2 ! general value");
        for (int l = 0; l < 12; ++l) f.line(std::to_string(in.ntimesg[l]));
        f.line("4 ! minor species");
        if (!f.close()) return GFM_E_IO;
    }
    return GFM_OK;
}
