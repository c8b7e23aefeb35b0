// model.cpp -- GAP XML reader and model set-up (host side).
//
// Reads the file format written by gap_fit and read by QUIP:
//   IPModel_GAP_read_params_xml (src/Potentials/IPModel_GAP.f95:618-944): GAP_params
//   (label, gap_version), GAP_data (e0 default, <e0 Z= value=/> per species);
//   gp_readXML (GAP, absent from the reference checkout; layout documented by
//   quippy/quippy/gap_tools.py:17-75 and tests/test_gapfit.py:154-170): gpSparse /
//   gpCoordinates (dimensions, signal_variance, signal_mean, covariance_type 1=ard_se
//   2=dot_product, zeta, sparseX_filename with M*D values one per line), <theta>,
//   <descriptor>, <sparseX alpha= sparseCutoff=/>.
// The SOAP radial basis set-up restates GAP's soap_initialise from the published
// construction (see soap_setup) and is computed here in FP64 once per model.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iterator>
#include <sstream>
#include <algorithm>
#include <memory>

#include "internal.h"

namespace gapgpu {

static thread_local std::string g_last_error;
void set_error(const std::string& msg) { g_last_error = msg; }
const char* last_error() { return g_last_error.c_str(); }

int SoapParams::n_pairs() const {
    int N = n_max * n_species;
    if (diagonal_radial) return n_max * n_species * (n_species + 1) / 2;
    return N * (N + 1) / 2;
}

// ------------------------------------------------------------------ minimal XML DOM
namespace {
struct XNode {
    std::string name, text;
    std::vector<std::pair<std::string, std::string>> attrs;
    std::vector<std::unique_ptr<XNode>> kids;
    const XNode* child(const std::string& n) const {
        for (auto& k : kids) if (k->name == n) return k.get();
        return nullptr;
    }
    bool attr(const std::string& n, std::string& v) const {
        for (auto& a : attrs) if (a.first == n) { v = a.second; return true; }
        return false;
    }
};

struct XParser {
    const char* s; size_t n, i = 0; std::string err;
    XParser(const char* s_, size_t n_) : s(s_), n(n_) {}
    bool eof() const { return i >= n; }
    bool starts(const char* p) const { size_t l = std::strlen(p); return i + l <= n && std::memcmp(s + i, p, l) == 0; }
    void skip_ws() { while (!eof() && std::isspace((unsigned char)s[i])) ++i; }
    static std::string unescape(const std::string& t) {
        std::string o; o.reserve(t.size());
        for (size_t k = 0; k < t.size(); ++k) {
            if (t[k] == '&') {
                size_t e = t.find(';', k);
                if (e != std::string::npos) {
                    std::string ent = t.substr(k + 1, e - k - 1);
                    if (ent == "lt") o += '<'; else if (ent == "gt") o += '>'; else if (ent == "amp") o += '&';
                    else if (ent == "quot") o += '"'; else if (ent == "apos") o += '\'';
                    else o += t.substr(k, e - k + 1);
                    k = e; continue;
                }
            }
            o += t[k];
        }
        return o;
    }
    bool skip_misc() {  // comments, PIs, doctype
        for (;;) {
            skip_ws();
            if (starts("<?")) { size_t e = std::string(s + i, n - i).find("?>"); if (e == std::string::npos) return false; i += e + 2; }
            else if (starts("<!--")) { size_t e = std::string(s + i, n - i).find("-->"); if (e == std::string::npos) return false; i += e + 3; }
            else if (starts("<!DOCTYPE")) { while (!eof() && s[i] != '>') ++i; ++i; }
            else return true;
        }
    }
    std::unique_ptr<XNode> element() {
        if (!skip_misc() || eof() || s[i] != '<') { err = "expected element"; return nullptr; }
        ++i;
        auto node = std::make_unique<XNode>();
        while (!eof() && !std::isspace((unsigned char)s[i]) && s[i] != '>' && s[i] != '/') node->name += s[i++];
        for (;;) {
            skip_ws();
            if (eof()) { err = "unterminated tag"; return nullptr; }
            if (s[i] == '/') { if (i + 1 < n && s[i + 1] == '>') { i += 2; return node; } err = "bad tag end"; return nullptr; }
            if (s[i] == '>') { ++i; break; }
            std::string an;
            while (!eof() && s[i] != '=' && !std::isspace((unsigned char)s[i])) an += s[i++];
            skip_ws();
            if (eof() || s[i] != '=') { err = "attribute without value: " + an; return nullptr; }
            ++i; skip_ws();
            char q = s[i];
            if (q != '"' && q != '\'') { err = "unquoted attribute " + an; return nullptr; }
            ++i;
            std::string v;
            while (!eof() && s[i] != q) v += s[i++];
            ++i;
            node->attrs.push_back({an, unescape(v)});
        }
        // content
        for (;;) {
            if (eof()) { err = "unterminated element " + node->name; return nullptr; }
            if (starts("</")) {
                i += 2;
                std::string en;
                while (!eof() && s[i] != '>') en += s[i++];
                ++i;
                while (!en.empty() && std::isspace((unsigned char)en.back())) en.pop_back();
                if (en != node->name) { err = "mismatched </" + en + "> for <" + node->name + ">"; return nullptr; }
                return node;
            }
            if (starts("<![CDATA[")) {
                size_t e = std::string(s + i, n - i).find("]]>");
                if (e == std::string::npos) { err = "unterminated CDATA"; return nullptr; }
                node->text.append(s + i + 9, e - 9);
                i += e + 3;
                continue;
            }
            if (starts("<!--")) { size_t e = std::string(s + i, n - i).find("-->"); if (e == std::string::npos) { err = "bad comment"; return nullptr; } i += e + 3; continue; }
            if (s[i] == '<') {
                auto k = element();
                if (!k) return nullptr;
                node->kids.push_back(std::move(k));
                continue;
            }
            size_t st = i;
            while (!eof() && s[i] != '<') ++i;
            node->text += unescape(std::string(s + st, i - st));
        }
    }
};

void find_all(const XNode* n, const std::string& name, std::vector<const XNode*>& out) {
    if (n->name == name) out.push_back(n);
    for (auto& k : n->kids) find_all(k.get(), name, out);
}

bool to_double(const std::string& v, double& d) {
    std::string t = v;
    for (auto& c : t) if (c == 'd' || c == 'D') c = 'e';  // Fortran exponent
    char* end = nullptr;
    d = std::strtod(t.c_str(), &end);
    return end != t.c_str();
}
std::vector<int> to_ints(const std::string& v) {
    std::vector<int> o;
    std::stringstream ss(v);
    std::string tok;
    while (ss >> tok) {
        for (auto& c : tok) if (c == ',') c = ' ';
        std::stringstream s2(tok);
        int x;
        while (s2 >> x) o.push_back(x);
    }
    return o;
}
bool to_bool(const std::string& v) {
    std::string u;
    for (char c : v) u += (char)std::toupper((unsigned char)c);
    return u == "T" || u == "TRUE" || u == ".TRUE." || u == "1";
}
}  // namespace

// key=value args_str parser (ParamReader.f95 semantics: values may be {..} or "..").
std::map<std::string, std::string> parse_args(const std::string& s) {
    std::map<std::string, std::string> out;
    size_t i = 0, n = s.size();
    while (i < n) {
        while (i < n && std::isspace((unsigned char)s[i])) ++i;
        if (i >= n) break;
        std::string key;
        while (i < n && s[i] != '=' && !std::isspace((unsigned char)s[i])) key += s[i++];
        size_t j = i;
        while (j < n && std::isspace((unsigned char)s[j])) ++j;
        if (j < n && s[j] == '=') {
            i = j + 1;
            while (i < n && std::isspace((unsigned char)s[i])) ++i;
            std::string v;
            if (i < n && (s[i] == '{' || s[i] == '"' || s[i] == '\'')) {
                char close = s[i] == '{' ? '}' : s[i];
                ++i;
                while (i < n && s[i] != close) v += s[i++];
                ++i;
            } else {
                while (i < n && !std::isspace((unsigned char)s[i])) v += s[i++];
            }
            out[key] = v;
        } else {
            out[key] = "T";  // bare word (descriptor name, "IP", "GAP")
        }
    }
    return out;
}

static double overlap_gauss(double a, double b, double al) {
    return std::exp(-al * (a * a + b * b)) * std::sqrt(2.0) * std::pow(al, 1.5) * (a + b) +
           al * std::exp(-0.5 * al * (a - b) * (a - b)) * std::sqrt(M_PI) * (1.0 + al * (a + b) * (a + b)) *
               (1.0 + std::erf(std::sqrt(al / 2.0) * (a + b)));
}

// SOAP radial basis (GAP soap_initialise restated): Gaussians exp(-alpha (r - r_b)^2),
// alpha = 1/(2 sigma^2), on r_b = b (rc + sigma sqrt(2 eps ln 10)) / n_max,
// b = 0..n_max-1 (eps = basis_error_exponent).  Neighbour densities are collocated
// on the grid; T = K^-1 L with K_ab = exp(-alpha (r_a - r_b)^2) and S = L L^T the
// analytic r^2-weighted overlap of the Gaussians, so that c = rho(grid) T are
// coefficients in an orthonormal radial basis.
void soap_setup(SoapParams& s) {
    const int n = s.n_max;
    s.alpha = 0.5 / (s.sigma * s.sigma);
    const double step = (s.rc + s.sigma * std::sqrt(2.0 * s.bee * std::log(10.0))) / n;
    s.rb.resize(n);
    for (int b = 0; b < n; ++b) s.rb[b] = step * b;
    std::vector<double> S(n * n), K(n * n), L(n * n, 0.0);
    for (int a = 0; a < n; ++a)
        for (int b = 0; b < n; ++b) {
            S[a * n + b] = overlap_gauss(s.rb[a], s.rb[b], s.alpha);
            K[a * n + b] = std::exp(-s.alpha * (s.rb[a] - s.rb[b]) * (s.rb[a] - s.rb[b]));
        }
    for (int j = 0; j < n; ++j) {
        double d = S[j * n + j];
        for (int k = 0; k < j; ++k) d -= L[j * n + k] * L[j * n + k];
        L[j * n + j] = std::sqrt(d);
        for (int i = j + 1; i < n; ++i) {
            double v = S[i * n + j];
            for (int k = 0; k < j; ++k) v -= L[i * n + k] * L[j * n + k];
            L[i * n + j] = v / L[j * n + j];
        }
    }
    // Solve K T = L (partial pivoting)
    std::vector<double> A = K, B = L;
    for (int c = 0; c < n; ++c) {
        int p = c;
        for (int r = c + 1; r < n; ++r) if (std::fabs(A[r * n + c]) > std::fabs(A[p * n + c])) p = r;
        if (p != c) for (int k = 0; k < n; ++k) { std::swap(A[c * n + k], A[p * n + k]); std::swap(B[c * n + k], B[p * n + k]); }
        for (int r = 0; r < n; ++r) {
            if (r == c) continue;
            double f = A[r * n + c] / A[c * n + c];
            if (f == 0.0) continue;
            for (int k = 0; k < n; ++k) { A[r * n + k] -= f * A[c * n + k]; B[r * n + k] -= f * B[c * n + k]; }
        }
    }
    s.T.assign(n * n, 0.0);
    for (int r = 0; r < n; ++r)
        for (int k = 0; k < n; ++k) s.T[r * n + k] = B[r * n + k] / A[r * n + r];
    // central atom: density at r=0 is exp(-alpha r_b^2) (l = 0 only), times Y_00
    s.centre_R.assign(n, 0.0);
    for (int nn = 0; nn < n; ++nn) {
        double R = 0;
        for (int a = 0; a < n; ++a) R += s.T[a * n + nn] * std::exp(-s.alpha * s.rb[a] * s.rb[a]);
        s.centre_R[nn] = s.cw * R * 0.5 / std::sqrt(M_PI);
    }
}

// Longest-processing-time assignment of the forward kernel's neighbour-function tasks to
// its 8 warps (the costs are relative step counts of the recurrences).
static void schedule_functions(const SoapParams& s, SoapConst& k) {
    const int L = s.l_max + 1, nm = s.n_max;
    struct Task { double cost; int code; };
    auto radial = [&](int a) { return s.rb[a] == 0.0 ? 2.0 : 4.0 + L; };
    auto ylm = [&](int m) { return 1.0 + 0.5 * m + 1.2 * (L - m); };
    auto assign = [](std::vector<Task> tasks, auto put) {
        std::stable_sort(tasks.begin(), tasks.end(), [](const Task& x, const Task& y) { return x.cost > y.cost; });
        double load[8] = {0};
        int used[8] = {0};
        for (const Task& t : tasks) {
            int w = -1;
            for (int i = 0; i < 8; ++i)
                if (used[i] < 8 && (w < 0 || load[i] < load[w])) w = i;
            put(w, used[w]++, t.code);
            load[w] += t.cost;
        }
    };
    std::memset(k.fsched, 0xff, sizeof k.fsched);
    std::vector<Task> f;
    for (int a = 0; a < nm; ++a) f.push_back({radial(a), a});
    for (int m = 0; m < L; ++m) f.push_back({ylm(m), nm + m});
    assign(f, [&](int w, int j, int code) { k.fsched[w][j] = (unsigned char)code; });
}

SoapConst soap_const(const Coordinate& c) {
    SoapConst k;
    std::memset(&k, 0, sizeof k);
    const SoapParams& s = c.soap;
    k.rc = s.rc; k.w = s.w; k.alpha = s.alpha; k.sigma0 = s.sigma0;
    k.l_max = s.l_max; k.n_max = s.n_max; k.n_species = s.n_species; k.n_pairs = s.n_pairs();
    k.dim = s.dim(); k.dpad = c.Dpad;
    k.ncomp = s.n_species * s.n_max * (s.l_max + 1) * (s.l_max + 1);
    k.normalise = s.normalise;
    for (int i = 0; i < MAX_SPECIES; ++i) k.species_Z[i] = i < s.n_species ? s.species_Z[i] : -1;
    for (int i = 0; i < s.n_max; ++i) { k.rb[i] = s.rb[i]; k.centre_R[i] = s.centre_R[i]; }
    for (int i = 0; i < s.n_max * s.n_max; ++i) k.T[i] = s.T[i];
    k.centre_all = s.central_all;
    schedule_functions(s, k);
    return k;
}

static int parse_soap(const std::map<std::string, std::string>& a, SoapParams& s) {
    auto get = [&](const char* k, const char* dflt) {
        auto it = a.find(k);
        return it == a.end() ? std::string(dflt) : it->second;
    };
    double v;
    if (!to_double(get("cutoff", "0"), s.rc) || s.rc <= 0) GG_FAIL(GAPGPU_ERR_XML, "soap: cutoff missing or not positive");
    to_double(get("cutoff_transition_width", "0.5"), s.w);
    std::string sig = a.count("atom_sigma") ? get("atom_sigma", "1.0") : get("atom_gaussian_width", "1.0");
    to_double(sig, s.sigma);
    to_double(get("central_weight", "1.0"), s.cw);
    to_double(get("covariance_sigma0", "0.0"), s.sigma0);
    to_double(get("basis_error_exponent", "10.0"), s.bee);
    s.l_max = std::atoi(get("l_max", "4").c_str());
    s.n_max = std::atoi(get("n_max", "4").c_str());
    s.n_species = std::atoi(get("n_species", "1").c_str());
    s.normalise = to_bool(get("normalise", "T"));
    s.diagonal_radial = to_bool(get("diagonal_radial", "F"));
    s.central_all = to_bool(get("central_reference_all_species", "F"));
    if (s.n_max < 1 || s.n_max > MAX_NMAX) GG_FAIL(GAPGPU_ERR_UNSUPPORTED, "soap: n_max outside 1..16");
    if (s.l_max < 0 || s.l_max > MAX_LMAX) GG_FAIL(GAPGPU_ERR_UNSUPPORTED, "soap: l_max outside 0..12");
    if (s.n_species < 1 || s.n_species > MAX_SPECIES) GG_FAIL(GAPGPU_ERR_UNSUPPORTED, "soap: n_species outside 1..8");
    if (s.diagonal_radial) GG_FAIL(GAPGPU_ERR_UNSUPPORTED, "soap: diagonal_radial=T is not supported");
    for (const char* k : {"average", "Z_mix", "R_mix", "sym_mix", "coupling", "K", "radial_enhancement", "compress_file",
                          "compress_mode"}) {
        auto it = a.find(k);
        if (it != a.end() && it->second != "F" && it->second != "0" && it->second != "none" && it->second != "")
            GG_FAIL(GAPGPU_ERR_UNSUPPORTED, std::string("soap: option ") + k + " is not supported");
    }
    if (a.count("cutoff_dexp") && std::atoi(get("cutoff_dexp", "0").c_str()) != 0)
        GG_FAIL(GAPGPU_ERR_UNSUPPORTED, "soap: cutoff_dexp != 0 is not supported");
    std::vector<int> sz = to_ints(get("species_Z", ""));
    if (sz.empty()) sz.assign(s.n_species, 0);
    if ((int)sz.size() < s.n_species) GG_FAIL(GAPGPU_ERR_XML, "soap: species_Z shorter than n_species");
    for (int i = 0; i < s.n_species; ++i) s.species_Z[i] = sz[i];
    std::vector<int> zc = to_ints(get("Z", "0"));
    s.n_Z = a.count("n_Z") ? std::atoi(get("n_Z", "1").c_str()) : (int)zc.size();
    if (s.n_Z < 1 || s.n_Z > MAX_CENTRE_Z || (int)zc.size() < s.n_Z) GG_FAIL(GAPGPU_ERR_XML, "soap: inconsistent n_Z / Z");
    for (int i = 0; i < s.n_Z; ++i) s.Z[i] = zc[i];
    soap_setup(s);
    (void)v;
    return GAPGPU_OK;
}

int parse_model(const char* xml, size_t len, const char* init_args, const char* base_dir, gapgpu_model& m) {
    if (!xml) GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_model_create: xml is NULL");
    std::map<std::string, std::string> ia = parse_args(init_args ? init_args : "");
    std::string label = ia.count("label") ? ia["label"] : "";
    if (ia.count("E_scale")) to_double(ia["E_scale"], m.E_scale);
    // the variance estimate is set up only when the init args name its regularisation
    // (IPModel_GAP.f95:170-171, :185-187)
    if (ia.count("gap_variance_regularisation")) {
        m.var_requested = true;
        if (!to_double(ia["gap_variance_regularisation"], m.var_reg) || !(m.var_reg >= 0))
            GG_FAIL(GAPGPU_ERR_ARG, "gap_variance_regularisation must be a non-negative number");
    }
    XParser p(xml, len);
    std::unique_ptr<XNode> root = p.element();
    if (!root) GG_FAIL(GAPGPU_ERR_XML, "GAP XML parse error: " + p.err);
    std::vector<const XNode*> gps;
    find_all(root.get(), "GAP_params", gps);
    const XNode* gp = nullptr;
    for (const XNode* g : gps) {
        std::string l;
        g->attr("label", l);
        if (label.empty() || l == label) { gp = g; m.label = l; break; }
    }
    if (!gp) GG_FAIL(GAPGPU_ERR_XML, "no GAP_params stanza with label '" + label + "'");
    std::string v;
    if (gp->attr("gap_version", v)) m.xml_version = std::atoi(v.c_str());
    if (const XNode* gd = gp->child("GAP_data")) {
        double d;
        if (gd->attr("e0", v) && to_double(v, d)) for (int z = 0; z < 128; ++z) m.e0[z] = d;
        for (auto& k : gd->kids) {
            if (k->name != "e0") continue;
            std::string zs, vs;
            if (!k->attr("Z", zs) || !k->attr("value", vs)) GG_FAIL(GAPGPU_ERR_XML, "e0 element without Z or value");
            int z = std::atoi(zs.c_str());
            if (z < 0 || z >= 128 || !to_double(vs, d)) GG_FAIL(GAPGPU_ERR_XML, "bad e0 entry");
            m.e0[z] = d;
        }
        if (gd->attr("do_pca", v) && to_bool(v)) GG_FAIL(GAPGPU_ERR_UNSUPPORTED, "GAP_data do_pca=T is not supported");
    }
    const XNode* sp = gp->child("gpSparse");
    if (!sp) GG_FAIL(GAPGPU_ERR_XML, "GAP_params without gpSparse");
    for (auto& gcp : sp->kids) {
        const XNode* gc = gcp.get();
        if (gc->name != "gpCoordinates") continue;
        Coordinate c;
        std::string a;
        if (!gc->attr("dimensions", a)) GG_FAIL(GAPGPU_ERR_XML, "gpCoordinates without dimensions");
        c.D = std::atoi(a.c_str());
        if (!gc->attr("covariance_type", a)) GG_FAIL(GAPGPU_ERR_XML, "gpCoordinates without covariance_type");
        c.cov = std::atoi(a.c_str());
        if (c.cov != COV_ARD_SE && c.cov != COV_DOT_PRODUCT)
            GG_FAIL(GAPGPU_ERR_UNSUPPORTED, "covariance_type " + a + " (only 1=ard_se, 2=dot_product)");
        if (!gc->attr("signal_variance", a) || !to_double(a, c.delta)) GG_FAIL(GAPGPU_ERR_XML, "missing signal_variance");
        if (gc->attr("signal_mean", a)) to_double(a, c.signal_mean);
        if (c.signal_mean != 0.0) GG_FAIL(GAPGPU_ERR_UNSUPPORTED, "non-zero signal_mean is not supported");
        if (gc->attr("zeta", a)) to_double(a, c.zeta);
        if (gc->attr("n_permutations", a) && std::atoi(a.c_str()) > 1)
            GG_FAIL(GAPGPU_ERR_UNSUPPORTED, "descriptor permutations > 1 are not supported");
        const XNode* dn = gc->child("descriptor");
        if (!dn) GG_FAIL(GAPGPU_ERR_XML, "gpCoordinates without descriptor");
        c.desc_str = dn->text;
        auto da = parse_args(c.desc_str);
        if (da.count("soap")) {
            c.type = DESC_SOAP;
            int rc = parse_soap(da, c.soap);
            if (rc) return rc;
            if (c.soap.dim() != c.D) GG_FAIL(GAPGPU_ERR_XML, "soap dimension mismatch with gpCoordinates dimensions");
        } else if (da.count("distance_2b")) {
            c.type = DESC_DISTANCE_2B;
            if (!to_double(da.count("cutoff") ? da["cutoff"] : "0", c.d2_rc) || c.d2_rc <= 0)
                GG_FAIL(GAPGPU_ERR_XML, "distance_2b: cutoff missing");
            if (da.count("cutoff_transition_width")) to_double(da["cutoff_transition_width"], c.d2_w);
            c.d2_Z1 = da.count("Z1") ? std::atoi(da["Z1"].c_str()) : 0;
            c.d2_Z2 = da.count("Z2") ? std::atoi(da["Z2"].c_str()) : 0;
            for (const char* k : {"exponents", "tail_range", "only_intra", "only_inter", "resid_name"})
                if (da.count(k) && !(da[k] == "F" || (std::string(k) == "exponents" && da[k] == "1")))
                    GG_FAIL(GAPGPU_ERR_UNSUPPORTED, std::string("distance_2b: option ") + k + " is not supported");
            if (c.D != 1) GG_FAIL(GAPGPU_ERR_XML, "distance_2b must have dimensions=1");
        } else {
            GG_FAIL(GAPGPU_ERR_UNSUPPORTED, "descriptor '" + c.desc_str.substr(0, 40) + "' is not supported (soap, distance_2b)");
        }
        if (c.cov == COV_ARD_SE) {
            const XNode* th = gc->child("theta");
            if (!th) GG_FAIL(GAPGPU_ERR_XML, "ard_se coordinate without theta");
            std::stringstream ss(th->text);
            std::string tok;
            double d;
            while (ss >> tok) if (to_double(tok, d)) c.theta.push_back(d);
            if ((int)c.theta.size() != c.D) GG_FAIL(GAPGPU_ERR_XML, "theta length != dimensions");
        }
        std::vector<const XNode*> sx;
        for (auto& k : gc->kids) if (k->name == "sparseX") sx.push_back(k.get());
        c.M = (int)sx.size();
        if (c.M == 0) GG_FAIL(GAPGPU_ERR_XML, "gpCoordinates without sparseX");
        c.alpha.resize(c.M);
        c.sc.assign(c.M, 1.0);
        for (int s = 0; s < c.M; ++s) {
            if (!sx[s]->attr("alpha", a) || !to_double(a, c.alpha[s])) GG_FAIL(GAPGPU_ERR_XML, "sparseX without alpha");
            if (sx[s]->attr("sparseCutoff", a)) to_double(a, c.sc[s]);
        }
        c.X.resize((size_t)c.M * c.D);
        if (gc->attr("sparseX_filename", a)) {
            std::string path = a;
            if (base_dir && *base_dir && !path.empty() && path[0] != '/') path = std::string(base_dir) + "/" + path;
            std::ifstream f(path, std::ios::binary);
            if (!f) GG_FAIL(GAPGPU_ERR_XML, "cannot open sparseX file " + path);
            std::string buf((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
            for (auto& ch : buf) if (ch == 'd' || ch == 'D') ch = 'e';  // Fortran exponents
            const char* q = buf.c_str();
            size_t k = 0;
            while (k < c.X.size()) {
                char* end = nullptr;
                double d = std::strtod(q, &end);
                if (end == q) break;
                c.X[k++] = d;
                q = end;
            }
            if (k != c.X.size()) GG_FAIL(GAPGPU_ERR_XML, "sparseX file " + path + " holds fewer than M*D values");
        } else {
            size_t k = 0;
            for (int s = 0; s < c.M; ++s) {
                std::stringstream ss(sx[s]->text);
                std::string tok;
                double d;
                while (ss >> tok && to_double(tok, d)) { if (k < c.X.size()) c.X[k] = d; ++k; }
            }
            if (k != c.X.size()) GG_FAIL(GAPGPU_ERR_XML, "inline sparseX values do not match M*D");
        }
        m.coords.push_back(std::move(c));
    }
    if (m.coords.empty()) GG_FAIL(GAPGPU_ERR_XML, "GAP model without gpCoordinates");
    m.cutoff = 0;
    for (auto& c : m.coords) m.cutoff = std::max(m.cutoff, c.cutoff());
    return GAPGPU_OK;
}

}  // namespace gapgpu
