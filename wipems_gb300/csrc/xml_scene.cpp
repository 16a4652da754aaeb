// openEMS XML input (the subset the engine covers) -> scene.
//
// openEMS reads one XML document (openEMS::ParseFDTDSetup, openems.cpp:756-
// 796): an <FDTD> element with the run settings, parsed by openEMS itself
// (Parse_XML_FDTDSetup, openems.cpp:798-936), and a <ContinuousStructure>
// element with the mesh, materials and probes, parsed by the CSXCAD library
// (ContinuousStructure::ReadFromXML, not part of the openEMS tree).  The
// matlab/python front ends write that document (matlab/WriteOpenEMS.m,
// InitFDTD.m, SetGaussExcite.m, SetBoundaryCond.m).
//
// Covered: <FDTD NumberOfTimesteps endCriteria OverSampling f_max>, its
// <Excitation> of Type 0 (Gaussian, f0 fc), 1 (sinusoid, f0), 2 (Dirac),
// 3 (step) or 10 (custom: Function f0), and <BoundaryCond> (numeric codes or
// PEC / PMC / MUR / PML_n, MUR_PhaseVelocity[_face]); the <RectilinearGrid DeltaUnit> with its X/Y/ZLines,
// <BackgroundMaterial>, and the properties Material, Metal, LumpedElement,
// Excitation, ProbeBox (voltage and current) and LorentzMaterial (order 1,
// electric and magnetic families),
// each with <Box> primitives (Priority, P1, P2).  Anything else that would
// change the simulation (other primitives, excitation signals, anisotropic
// or weighted materials, cylindrical coordinates) is
// refused with FDTD_ERR_UNSUPPORTED and a message naming it; purely visual
// elements (colours) are ignored.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "fdtd_host.h"

namespace wipems {
namespace {

// ------------------------------------------------------------ tiny XML DOM
struct XNode {
    std::string name;
    std::vector<std::pair<std::string, std::string>> attrs;
    std::vector<XNode> kids;
    std::string text;
    const std::string* attr(const char* k) const {
        for (const auto& a : attrs)
            if (a.first == k) return &a.second;
        return nullptr;
    }
    const XNode* child(const char* n) const {
        for (const auto& c : kids)
            if (c.name == n) return &c;
        return nullptr;
    }
};

struct XParser {
    const std::string& s;
    size_t i = 0;
    std::string err;
    explicit XParser(const std::string& src) : s(src) {}

    bool fail(const std::string& m) {
        if (err.empty()) err = m + " (at byte " + std::to_string(i) + ")";
        return false;
    }
    void ws() {
        while (i < s.size() && std::isspace((unsigned char)s[i])) ++i;
    }
    bool starts(const char* p) const { return s.compare(i, std::strlen(p), p) == 0; }
    static std::string unescape(const std::string& v) {
        std::string o;
        for (size_t k = 0; k < v.size(); ++k) {
            if (v[k] != '&') {
                o += v[k];
                continue;
            }
            const size_t e = v.find(';', k);
            if (e == std::string::npos) {
                o += v[k];
                continue;
            }
            const std::string ent = v.substr(k + 1, e - k - 1);
            if (ent == "lt") o += '<';
            else if (ent == "gt") o += '>';
            else if (ent == "amp") o += '&';
            else if (ent == "quot") o += '"';
            else if (ent == "apos") o += '\'';
            else if (!ent.empty() && ent[0] == '#') o += (char)std::strtol(ent.c_str() + 1 + (ent[1] == 'x'), nullptr, ent[1] == 'x' ? 16 : 10);
            else o += "&" + ent + ";";
            k = e;
        }
        return o;
    }
    // skips declarations, processing instructions and comments
    bool misc() {
        for (;;) {
            ws();
            if (starts("<?")) {
                const size_t e = s.find("?>", i);
                if (e == std::string::npos) return fail("unterminated <?");
                i = e + 2;
            } else if (starts("<!--")) {
                const size_t e = s.find("-->", i);
                if (e == std::string::npos) return fail("unterminated comment");
                i = e + 3;
            } else if (starts("<!")) {
                const size_t e = s.find('>', i);
                if (e == std::string::npos) return fail("unterminated <!");
                i = e + 1;
            } else {
                return true;
            }
        }
    }
    bool name(std::string& out) {
        const size_t b = i;
        while (i < s.size() && (std::isalnum((unsigned char)s[i]) || s[i] == '_' || s[i] == '-' || s[i] == ':' ||
                                s[i] == '.'))
            ++i;
        if (i == b) return fail("expected a name");
        out = s.substr(b, i - b);
        return true;
    }
    bool element(XNode& n, int depth) {
        if (depth > 64) return fail("elements nested too deeply");
        if (i >= s.size() || s[i] != '<') return fail("expected '<'");
        ++i;
        if (!name(n.name)) return false;
        for (;;) {
            ws();
            if (i >= s.size()) return fail("unterminated tag <" + n.name + ">");
            if (starts("/>")) {
                i += 2;
                return true;
            }
            if (s[i] == '>') {
                ++i;
                break;
            }
            std::string k;
            if (!name(k)) return false;
            ws();
            if (i >= s.size() || s[i] != '=') return fail("expected '=' after attribute " + k);
            ++i;
            ws();
            if (i >= s.size() || (s[i] != '"' && s[i] != '\'')) return fail("expected a quoted value for " + k);
            const char q = s[i++];
            const size_t e = s.find(q, i);
            if (e == std::string::npos) return fail("unterminated attribute " + k);
            n.attrs.emplace_back(k, unescape(s.substr(i, e - i)));
            i = e + 1;
        }
        // content
        for (;;) {
            const size_t lt = s.find('<', i);
            if (lt == std::string::npos) return fail("unterminated element <" + n.name + ">");
            n.text += unescape(s.substr(i, lt - i));
            i = lt;
            if (starts("<!--")) {
                const size_t e = s.find("-->", i);
                if (e == std::string::npos) return fail("unterminated comment");
                i = e + 3;
                continue;
            }
            if (starts("<![CDATA[")) {
                const size_t e = s.find("]]>", i);
                if (e == std::string::npos) return fail("unterminated CDATA");
                n.text += s.substr(i + 9, e - i - 9);
                i = e + 3;
                continue;
            }
            if (starts("</")) {
                i += 2;
                std::string close;
                if (!name(close)) return false;
                if (close != n.name) return fail("</" + close + "> closes <" + n.name + ">");
                ws();
                if (i >= s.size() || s[i] != '>') return fail("expected '>'");
                ++i;
                return true;
            }
            n.kids.emplace_back();
            if (!element(n.kids.back(), depth + 1)) return false;
        }
    }
    bool document(XNode& root) {
        if (!misc()) return false;
        if (!element(root, 0)) return false;
        return misc();
    }
};

// ------------------------------------------------------------ value parsing
bool to_double(const std::string& t, double& v) {
    std::string u;
    for (char c : t)
        if (!std::isspace((unsigned char)c)) u += (char)std::tolower((unsigned char)c);
    if (u == "nan") {
        v = NAN;
        return true;
    }
    if (u == "inf" || u == "+inf") {
        v = INFINITY;
        return true;
    }
    if (u == "-inf") {
        v = -INFINITY;
        return true;
    }
    char* e = nullptr;
    v = std::strtod(u.c_str(), &e);
    return !u.empty() && e && *e == 0;
}

bool list(const std::string& t, std::vector<double>& out) {
    out.clear();
    std::string cur;
    auto flush = [&]() -> bool {
        if (cur.empty()) return true;
        double v;
        if (!to_double(cur, v)) return false;
        out.push_back(v);
        cur.clear();
        return true;
    };
    for (char c : t) {
        if (c == ',' || c == ';' || std::isspace((unsigned char)c)) {
            if (!flush()) return false;
        } else {
            cur += c;
        }
    }
    return flush();
}

struct Loader {
    std::string err;
    int code = FDTD_OK;
    bool bad(int c, const std::string& m) {
        if (code == FDTD_OK) {
            code = c;
            err = m;
        }
        return false;
    }
    bool num(const XNode& n, const char* k, double& v, double dflt) {
        const std::string* a = n.attr(k);
        if (!a) {
            v = dflt;
            return true;
        }
        if (!to_double(*a, v)) return bad(FDTD_ERR_ARG, "<" + n.name + " " + k + "=\"" + *a + "\">: not a number");
        return true;
    }
    // isotropic value of a scalar or "a,b,c" attribute
    bool iso(const XNode& n, const char* k, double& v, double dflt) {
        const std::string* a = n.attr(k);
        if (!a) {
            v = dflt;
            return true;
        }
        std::vector<double> l;
        if (!list(*a, l) || l.empty()) return bad(FDTD_ERR_ARG, "<" + n.name + " " + k + "=\"" + *a + "\">: not a number");
        for (double x : l)
            if (!(x == l[0])) return bad(FDTD_ERR_UNSUPPORTED, "anisotropic " + std::string(k) + " in <" + n.name + ">");
        v = l[0];
        return true;
    }
    bool point(const XNode& p, double c[3]) {
        const char* ax[3] = {"X", "Y", "Z"};
        for (int a = 0; a < 3; ++a) {
            const std::string* v = p.attr(ax[a]);
            if (!v || !to_double(*v, c[a])) return bad(FDTD_ERR_ARG, "<" + p.name + ">: coordinate " + ax[a] + " missing");
        }
        return true;
    }
};

struct Box {
    int priority;
    double a[3], b[3];
};

}  // namespace
}  // namespace wipems

using namespace wipems;

extern "C" {

int fdtd_scene_load_xml(const char* text, fdtd_scene_t* out, fdtd_xml_info* info) {
    if (!text || !out) {
        set_error("fdtd_scene_load_xml: null argument");
        return FDTD_ERR_ARG;
    }
    const std::string src(text);
    XNode root;
    XParser P(src);
    if (!P.document(root)) {
        set_error("openEMS XML: " + P.err);
        return FDTD_ERR_ARG;
    }
    Loader L;
    if (root.name != "openEMS") {
        set_error("openEMS XML: the root element is <" + root.name + ">, not <openEMS>");
        return FDTD_ERR_ARG;
    }
    const XNode* fdtd = root.child("FDTD");
    const XNode* csx = root.child("ContinuousStructure");
    if (!fdtd || !csx) {
        set_error("openEMS XML: <FDTD> and <ContinuousStructure> are required (openems.cpp:779-792)");
        return FDTD_ERR_ARG;
    }
    fdtd_xml_info inf;
    std::memset(&inf, 0, sizeof(inf));
    // ---- <FDTD> (openems.cpp:798-936)
    double d = 0;
    L.num(*fdtd, "NumberOfTimesteps", d, 0);
    inf.nr_ts = d < 0 ? 0u : (uint32_t)std::min(d, 4294967295.0);
    L.num(*fdtd, "endCriteria", d, 0);
    inf.end_crit = d == 0 ? 1e-6 : d;
    L.num(*fdtd, "OverSampling", d, 0);
    inf.oversampling = d > 1 ? (uint32_t)d : 0u;
    L.num(*fdtd, "CylinderCoords", d, 0);
    if (d == 1) L.bad(FDTD_ERR_UNSUPPORTED, "cylindrical coordinates (CylinderCoords=1)");
    for (const char* k : {"TimeStepMethod", "TimeStep", "TimeStepFactor", "MaxTime", "CellConstantMaterial"})
        if (fdtd->attr(k)) L.bad(FDTD_ERR_UNSUPPORTED, std::string("<FDTD ") + k + ">");
    const XNode* exc = fdtd->child("Excitation");
    if (!exc) L.bad(FDTD_ERR_ARG, "<FDTD> has no <Excitation> (openems.cpp:892-896)");
    // the signal (openems.cpp:898-926): Type 0 Gaussian (f0, fc), 1 sinusoid
    // (f0), 2 Dirac and 3 step (<FDTD f_max>), 10 custom (Function, f0,
    // <FDTD f_max>)
    double f0 = 0, fc = 0, f_max = 0;
    std::string function;
    if (exc) {
        L.num(*exc, "Type", d, -1);
        inf.excite_type = (int)d;
        if (((int)d < 0 || (int)d > 3) && (int)d != 10)
            L.bad(FDTD_ERR_UNSUPPORTED, "excitation Type " + std::to_string((int)d) +
                                            " (Gaussian 0, sinusoid 1, Dirac 2, step 3 and custom 10 are covered)");
        if ((int)d <= 1 || (int)d == 10) L.num(*exc, "f0", f0, 0);
        if ((int)d == 0) L.num(*exc, "fc", fc, 0);
        if ((int)d >= 2) L.num(*fdtd, "f_max", f_max, 0);
        if ((int)d == 10) {
            if (exc->attr("Function")) function = *exc->attr("Function");
            else L.bad(FDTD_ERR_ARG, "<Excitation Type=\"10\"> needs a Function attribute");
        }
    }
    inf.f0 = f0;
    inf.fc = fc;
    int bc[6] = {0, 0, 0, 0, 0, 0};
    uint32_t pml[6] = {8, 8, 8, 8, 8, 8};  // openEMS's default for every face (openems.cpp:101)
    const XNode* bcn = fdtd->child("BoundaryCond");
    if (!bcn) L.bad(FDTD_ERR_ARG, "<FDTD> has no <BoundaryCond> (openems.cpp:835-840)");
    const char* bnames[6] = {"xmin", "xmax", "ymin", "ymax", "zmin", "zmax"};
    for (int n = 0; bcn && n < 6; ++n) {
        const std::string* v = bcn->attr(bnames[n]);
        if (!v) continue;  // the reference warns and keeps PEC
        double code;
        if (to_double(*v, code)) {
            bc[n] = (int)code;
        } else if (*v == "PEC") {
            bc[n] = 0;
        } else if (*v == "PMC") {
            bc[n] = 1;
        } else if (*v == "MUR") {
            bc[n] = 2;
        } else if (v->compare(0, 4, "PML_") == 0) {
            bc[n] = 3;
            pml[n] = (uint32_t)std::atoi(v->c_str() + 4);
        }  // else: the reference warns and keeps PEC
    }
    // Mur phase velocities (openems.cpp:882-890)
    double vph[6] = {0, 0, 0, 0, 0, 0};
    if (bcn) {
        double v;
        L.num(*bcn, "MUR_PhaseVelocity", v, 0);
        for (int n = 0; n < 6; ++n) vph[n] = v;
        for (int n = 0; n < 6; ++n) {
            const std::string k = std::string("MUR_PhaseVelocity_") + bnames[n];
            if (bcn->attr(k.c_str())) L.num(*bcn, k.c_str(), vph[n], 0);
        }
    }
    // ---- <ContinuousStructure>: grid
    const XNode* grid = csx->child("RectilinearGrid");
    if (!grid) {
        set_error("openEMS XML: <ContinuousStructure> has no <RectilinearGrid>");
        return FDTD_ERR_ARG;
    }
    double unit = 1;
    L.num(*grid, "DeltaUnit", unit, 1);
    L.num(*grid, "CoordSystem", d, 0);
    if (d != 0) L.bad(FDTD_ERR_UNSUPPORTED, "cylindrical RectilinearGrid");
    std::vector<double> lines[3];
    const char* ln[3] = {"XLines", "YLines", "ZLines"};
    for (int a = 0; a < 3; ++a) {
        const XNode* l = grid->child(ln[a]);
        if (!l || !list(l->text, lines[a])) {
            set_error(std::string("openEMS XML: <") + ln[a] + "> missing or not a number list");
            return FDTD_ERR_ARG;
        }
        std::sort(lines[a].begin(), lines[a].end());  // CSRectGrid keeps lines sorted and unique
        lines[a].erase(std::unique(lines[a].begin(), lines[a].end()), lines[a].end());
    }
    if (L.code) {
        set_error("openEMS XML: " + L.err);
        return L.code;
    }
    fdtd_scene_t sc = nullptr;
    int rc = fdtd_scene_create(lines[0].data(), (uint32_t)lines[0].size(), lines[1].data(), (uint32_t)lines[1].size(),
                               lines[2].data(), (uint32_t)lines[2].size(), unit, &sc);
    if (rc) return rc;
    auto fail = [&](int c, const std::string& m) {
        fdtd_scene_destroy(sc);
        set_error("openEMS XML: " + m);
        return c;
    };
    if (const XNode* bg = csx->child("BackgroundMaterial")) {
        double e, m, k, s;
        L.num(*bg, "Epsilon", e, 1);
        L.num(*bg, "Mue", m, 1);
        L.num(*bg, "Kappa", k, 0);
        L.num(*bg, "Sigma", s, 0);
        if ((rc = fdtd_scene_set_background(sc, e, m, k, s))) return fail(rc, "background material");
    }
    if ((rc = fdtd_scene_set_boundary(sc, bc, pml))) return fail(rc, "boundary conditions");
    if ((rc = fdtd_scene_set_mur_velocity(sc, vph))) return fail(rc, "Mur phase velocity");
    if (inf.excite_type == 0 && (rc = fdtd_scene_set_gauss_excite(sc, f0, fc, inf.nr_ts)))
        return fail(rc, "Gaussian excitation");
    if (inf.excite_type == 1 && (rc = fdtd_scene_set_sinus_excite(sc, f0, inf.nr_ts)))
        return fail(rc, "sinusoidal excitation");
    if (inf.excite_type == 2 && (rc = fdtd_scene_set_dirac_excite(sc, f_max, inf.nr_ts)))
        return fail(rc, "Dirac excitation");
    if (inf.excite_type == 3 && (rc = fdtd_scene_set_step_excite(sc, f_max, inf.nr_ts)))
        return fail(rc, "step excitation");
    if (inf.excite_type == 10 && (rc = fdtd_scene_set_custom_excite(sc, function.c_str(), f0, f_max, inf.nr_ts)))
        return fail(rc, "custom excitation");
    if (inf.oversampling && (rc = fdtd_scene_set_oversampling(sc, inf.oversampling))) return fail(rc, "OverSampling");
    // ---- properties
    const XNode* props = csx->child("Properties");
    for (size_t pi = 0; props && pi < props->kids.size(); ++pi) {
        const XNode& p = props->kids[pi];
        const std::string pname = p.attr("Name") ? *p.attr("Name") : p.name;
        // boxes of this property
        std::vector<Box> boxes;
        if (const XNode* prims = p.child("Primitives")) {
            for (const XNode& g : prims->kids) {
                if (g.name != "Box") {
                    L.bad(FDTD_ERR_UNSUPPORTED, "primitive <" + g.name + "> of property '" + pname + "' (only <Box>)");
                    continue;
                }
                Box b;
                double pr;
                L.num(g, "Priority", pr, 0);
                b.priority = (int)pr;
                const XNode* p1 = g.child("P1");
                const XNode* p2 = g.child("P2");
                if (!p1 || !p2) {
                    L.bad(FDTD_ERR_ARG, "<Box> of '" + pname + "' needs <P1> and <P2>");
                    continue;
                }
                if (g.child("Transformation")) L.bad(FDTD_ERR_UNSUPPORTED, "transformed <Box> of '" + pname + "'");
                if (L.point(*p1, b.a) && L.point(*p2, b.b)) boxes.push_back(b);
            }
        }
        if (L.code) return fail(L.code, L.err);
        const XNode* pp = p.child("Property");
        static const XNode empty;
        const XNode& prop = pp ? *pp : empty;
        if (p.child("Weight")) {
            // weighting functions (fparser strings); all-1 weights are harmless
            for (const auto& a : p.child("Weight")->attrs) {
                double w;
                if (!to_double(a.second, w) || w != 1) L.bad(FDTD_ERR_UNSUPPORTED, "material weighting functions of '" + pname + "'");
            }
        }
        if (p.name == "Material" || p.name == "LorentzMaterial") {
            double e, m, k, s;
            L.iso(prop, "Epsilon", e, 1);
            L.iso(prop, "Mue", m, 1);
            L.iso(prop, "Kappa", k, 0);
            L.iso(prop, "Sigma", s, 0);
            double pf = 0, rt = 0, lf = 0, mpf = 0, mrt = 0, mlf = 0;
            if (p.name == "LorentzMaterial") {
                L.num(p, "Order", d, 1);
                if (d > 1) L.bad(FDTD_ERR_UNSUPPORTED, "dispersion Order " + std::to_string((int)d) + " of '" + pname + "'");
                L.iso(prop, "EpsilonPlasmaFrequency", pf, 0);
                L.iso(prop, "EpsilonRelaxTime", rt, 0);
                L.iso(prop, "EpsilonLorPoleFrequency", lf, 0);
                L.iso(prop, "MuePlasmaFrequency", mpf, 0);
                L.iso(prop, "MueRelaxTime", mrt, 0);
                L.iso(prop, "MueLorPoleFrequency", mlf, 0);
            }
            if (L.code) return fail(L.code, L.err);
            for (const Box& b : boxes) {
                rc = p.name == "Material"
                         ? fdtd_scene_add_material(sc, b.priority, b.a, b.b, e, k, m, s)
                         : fdtd_scene_add_lorentz_material(sc, b.priority, b.a, b.b, e, k, m, s, 1, &pf, &rt, &lf,
                                                           &mpf, &mrt, &mlf);
                if (rc) return fail(rc, "property '" + pname + "'");
                ++inf.num_boxes;
            }
        } else if (p.name == "Metal") {
            for (const Box& b : boxes) {
                if ((rc = fdtd_scene_add_metal(sc, b.priority, b.a, b.b))) return fail(rc, "metal '" + pname + "'");
                ++inf.num_boxes;
            }
        } else if (p.name == "LumpedElement") {
            double dir, R, C, Lh, caps;
            L.num(p, "Direction", dir, -1);
            L.num(p, "R", R, NAN);
            L.num(p, "C", C, NAN);
            L.num(p, "L", Lh, NAN);
            L.num(p, "Caps", caps, 1);
            double type;
            L.num(p, "LEtype", type, FDTD_LE_PARALLEL);  // -1 invalid, 0 parallel, 1 series
            if (type != FDTD_LE_INVALID && type != FDTD_LE_PARALLEL && type != FDTD_LE_SERIES)
                L.bad(FDTD_ERR_ARG, "<LumpedElement LEtype> of '" + pname + "'");
            if (L.code) return fail(L.code, L.err);
            for (const Box& b : boxes) {
                if ((rc = fdtd_scene_add_lumped_rlc(sc, b.priority, b.a, b.b, (int)dir, (int)type,
                                                    std::isnan(R) ? -1.0 : R, std::isnan(Lh) ? -1.0 : Lh,
                                                    std::isnan(C) ? -1.0 : C, caps != 0)))
                    return fail(rc, "lumped element '" + pname + "'");
                ++inf.num_boxes;
            }
        } else if (p.name == "Excitation") {
            double type, delay;
            L.num(p, "Type", type, 0);
            L.num(p, "Delay", delay, 0);
            std::vector<double> v;
            const std::string* ex = p.attr("Excite");
            if (!ex || !list(*ex, v) || v.size() != 3) L.bad(FDTD_ERR_ARG, "<Excitation Excite=\"x,y,z\"> of '" + pname + "'");
            if (type < 0 || type > 3) L.bad(FDTD_ERR_UNSUPPORTED, "excitation type " + std::to_string((int)type) + " of '" + pname + "'");
            if (L.code) return fail(L.code, L.err);
            for (const Box& b : boxes) {
                if ((rc = fdtd_scene_add_excitation(sc, b.priority, b.a, b.b, (int)type, v.data(), delay)))
                    return fail(rc, "excitation '" + pname + "'");
                ++inf.num_boxes;
            }
        } else if (p.name == "ProbeBox") {
            double type, weight, nd;
            L.num(p, "Type", type, 0);
            L.num(p, "Weight", weight, 1);
            L.num(p, "NormDir", nd, -1);
            if (type < 0 || type > 3) {  // mode-match and other probes
                ++inf.skipped;
                continue;
            }
            for (const Box& b : boxes) {
                if ((rc = fdtd_scene_add_probe(sc, (int)type, b.a, b.b, weight, (int)nd)))
                    return fail(rc, "probe '" + pname + "'");
                ++inf.num_probes;
            }
        } else if (p.name == "DumpBox") {
            // time-domain E / H dumps are recorded for the caller (they do not
            // change the fields); other dump types are skipped
            double type, mode, ftype;
            L.num(p, "DumpType", type, 0);
            L.num(p, "DumpMode", mode, 0);
            L.num(p, "FileType", ftype, 0);
            std::vector<double> sub;
            const std::string* ss = p.attr("SubSampling");
            if (ss && (!list(*ss, sub) || sub.size() != 3)) L.bad(FDTD_ERR_ARG, "<DumpBox SubSampling> of '" + pname + "'");
            if (L.code) return fail(L.code, L.err);
            if ((type != 0 && type != 1) || mode < 0 || mode > 2) {
                ++inf.skipped;
                continue;
            }
            for (const Box& b : boxes) {
                DumpSpec d;
                d.name = pname;
                d.field = (int)type;
                d.interp = (int)mode;
                d.file_type = (int)ftype;
                for (int a = 0; a < 3; ++a) {
                    d.start[a] = b.a[a];
                    d.stop[a] = b.b[a];
                    d.step[a] = ss ? (uint32_t)std::max(1.0, sub[a]) : 1u;
                }
                sc->dumps.push_back(d);
            }
        } else if (p.name == "DebyeMaterial" || p.name == "ConductingSheet" || p.name == "Resistance") {
            return fail(FDTD_ERR_UNSUPPORTED, "property <" + p.name + "> ('" + pname + "')");
        } else {
            return fail(FDTD_ERR_UNSUPPORTED, "property <" + p.name + "> ('" + pname + "')");
        }
        ++inf.num_properties;
    }
    if (info) *info = inf;
    *out = sc;
    return FDTD_OK;
}

int fdtd_scene_load_xml_file(const char* path, fdtd_scene_t* out, fdtd_xml_info* info) {
    if (!path || !out) {
        set_error("fdtd_scene_load_xml_file: null argument");
        return FDTD_ERR_ARG;
    }
    std::ifstream f(path, std::ios::binary);
    if (!f) {
        set_error(std::string("fdtd_scene_load_xml_file: cannot open ") + path);
        return FDTD_ERR_ARG;
    }
    std::stringstream ss;
    ss << f.rdbuf();
    const std::string text = ss.str();
    return fdtd_scene_load_xml(text.c_str(), out, info);
}

}  // extern "C"
