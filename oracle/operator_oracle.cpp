// ORACLE -- test infrastructure only.  Nothing in the product links or calls
// this file; tests/, __graft_entry__.smoke() and bench.py's CPU legs use it
// as the checker of the product's operator build and as the operator of the
// timed CPU reference.
//
// A second, independent CPU restatement of openEMS's operator build, written
// from the reference sources and structured like them: every coefficient is
// computed edge by edge through the same member functions the reference calls
// (material lookups at coordinates, not the product's per-line sampling), in
// the reference's order of double operations, stored as float where the
// reference stores FDTD_FLOAT.  Citations relative to the reference project:
//
//   mesh helpers GetDiscLine/GetDiscDelta/GetEdgeLength/GetNodeWidth/
//     GetNodeArea/GetYeeCoords          FDTD/operator.cpp:136-242, operator.h:126-150
//   SnapToMeshLine/SnapToMesh/SnapBox2Mesh  FDTD/operator.cpp:244-345
//   GetPrimitivesBoundBox                FDTD/operator.cpp:1760-1778
//   CalcECOperator (sequence)            FDTD/operator.cpp:973-1084
//   Calc_EC_Range / Calc_ECPos           FDTD/operator.cpp:1780-1803, 1176-1224
//   GetRawDiscDelta / GetMaterial        FDTD/operator.cpp:1226-1236, 1251-1298
//   AverageMatQuarterCell                FDTD/operator.cpp:1406-1518
//   Calc_ECOperatorPos                   FDTD/operator.cpp:943-971
//   ApplyElectricBC / ApplyMagneticBC    FDTD/operator.cpp:1086-1174
//   CalcPEC_Range                        FDTD/operator.cpp:1986-2020
//   Calc_LumpedElements (parallel RC)    FDTD/operator.cpp:1535-1712, IsLEparRC :1714-1724
//   CalcTimestep_Var3 (+ AdrOp reflect)  FDTD/operator.cpp:1897-1971, tools/AdrOp.cpp:183-222,327-386
//   extension order                      openems.cpp:1041-1096, 380-404
//   Operator_Ext_Excitation::BuildExtension  FDTD/extensions/operator_ext_excitation.cpp:101-285
//   Operator_Ext_Mur_ABC::SetDirection/BuildExtension  extensions/operator_ext_mur_abc.cpp:88-195
//     (start timestep: extensions/engine_ext_mur_abc.cpp:43-58)
//   Operator_Ext_UPML::Create_UPML / CalcGradingKappa / BuildExtension
//                                        extensions/operator_ext_upml.cpp:31,77-255,289-466
//   Operator_Ext_LorentzMaterial::BuildExtension  extensions/operator_ext_lorentzmaterial.cpp:117-414
//   Operator_Ext_LumpedRLC::BuildExtension   extensions/operator_ext_lumpedRLC.cpp:112-486
//   Excitation::CalcGaussianPulsExcitation   FDTD/excitation.cpp:151-177
//   Excitation::CalcSinusExcitation, CalcDiracPulsExcitation,
//   CalcStepExcitation                       FDTD/excitation.cpp:179-218, 273-295
//   periodic-signal timestep                 FDTD/operator.cpp:999-1007
//   CalcNyquistNum                       tools/useful.cpp:30-36
//   probe snapping: openEMS::SetupProcessing openems.cpp:470-540,
//     Processing::DefineStartStopCoord Common/processing.cpp:180-189,
//     ProcessVoltage Common/processvoltage.cpp:37-41,
//     ProcessCurrent Common/processcurrent.cpp:22-91, SetProcessInterval
//     Common/processing.cpp:206-209
//
// Third-party stand-in (CSXCAD is not part of the reference tree): each box is
// its own property; a lookup takes the primitives of the requested types,
// keeps those whose box holds the coordinate (bounds inclusive), and returns
// the one of highest priority, the first added on a tie
// (ContinuousStructure::GetPropertyByCoordPriority).  Material getters return
// the box's constant values (no weighting functions).  The UPML grading
// function, parsed by fparser in the reference, is evaluated as the C++
// expression of its default string.
#include <algorithm>
#include <cctype>
#include <climits>
#include <cstdlib>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../include/wipems_fdtd.h"

extern "C" {

// One box of the scene (kinds: 1 material, 2 metal, 3 lumped element,
// 4 excitation, 5 probe).  A material with disp_order > 0 is a
// Lorentz/Drude material (CSPropLorentzMaterial).
typedef struct {
    int kind;
    int priority;
    double start[3], stop[3];
    double eps, kappa, mue, sigma;
    int disp_order;
    double eps_plasma_f[4], eps_relax_t[4], eps_pole_f[4];
    double mue_plasma_f[4], mue_relax_t[4], mue_pole_f[4];
    int ny, le_type;
    double R, C, L;
    int caps;
    int exc_type;
    double exc_vec[3];
    double delay;
    int probe_type;
    double weight;
    int norm_dir;
} oracle_prim;

typedef struct {
    const double* lines[3];
    uint32_t num_lines[3];
    double unit;
    double bg_eps, bg_mue, bg_kappa, bg_sigma;
    int bc[6];
    uint32_t pml_size[6];
    double mur_vph[6];
    double f0, fc;
    uint32_t nr_ts;
    uint32_t oversampling;
    uint32_t num_prims;
    const oracle_prim* prims;
    int excite_type;  // Excitation::ExciteTypes: 0 Gaussian, 1 sinusoid, 2 Dirac, 3 step, 10 custom
    double f_max;
    const char* function;  // the custom signal (a function of t)
} oracle_scene;

typedef struct {
    uint32_t num_lines[3];
    double dT;
    uint32_t nyquist, probe_interval, signal_length, max_excite_ts;
    uint32_t num_probes;
} oracle_op_info;

}  // extern "C"

namespace {

constexpr double kEps0 = 8.85418781762e-12;  // tools/constants.h:23-27
constexpr double kMue0 = 1.256637062e-6;
constexpr double kC0 = 299792458;
constexpr double kZ0 = 376.730313461;
constexpr double kPI = 3.141592653589793238462643383279;

enum { T_MATERIAL = 1, T_METAL = 2, T_LUMPED = 4, T_EXCITATION = 8, T_PROBE = 16 };

int prim_type(const oracle_prim& p) {
    switch (p.kind) {
        case 1: return T_MATERIAL;
        case 2: return T_METAL;
        case 3: return T_LUMPED;
        case 4: return T_EXCITATION;
        case 5: return T_PROBE;
    }
    return 0;
}

struct Csx {
    std::vector<oracle_prim> P;
    std::vector<double> lo[3], hi[3];

    void init() {
        for (int n = 0; n < 3; ++n) {
            lo[n].resize(P.size());
            hi[n].resize(P.size());
            for (size_t i = 0; i < P.size(); ++i) {
                lo[n][i] = std::fmin(P[i].start[n], P[i].stop[n]);
                hi[n][i] = std::fmax(P[i].start[n], P[i].stop[n]);
            }
        }
    }
    bool inside(size_t i, const double* c) const {
        for (int n = 0; n < 3; ++n)
            if (c[n] < lo[n][i] || c[n] > hi[n][i]) return false;
        return true;
    }
    // ContinuousStructure::GetPrimitivesByBoundBox: primitives of the types
    // whose box meets the bound box [bb[0],bb[1]] x [bb[2],bb[3]] x [bb[4],bb[5]]
    std::vector<int> by_bound_box(const double* bb, int mask) const {
        std::vector<int> out;
        for (size_t i = 0; i < P.size(); ++i) {
            if (!(prim_type(P[i]) & mask)) continue;
            bool meet = true;
            for (int n = 0; n < 3 && meet; ++n)
                if (hi[n][i] < bb[2 * n] || lo[n][i] > bb[2 * n + 1]) meet = false;
            if (meet) out.push_back((int)i);
        }
        return out;
    }
    // ContinuousStructure::GetPropertyByCoordPriority over a primitive list
    int by_coord_priority(const double* c, const std::vector<int>& list) const {
        int win = -1;
        for (int i : list)
            if (inside((size_t)i, c) && (win < 0 || P[i].priority > P[win].priority)) win = i;
        return win;
    }
    std::vector<int> by_type(int mask) const {
        std::vector<int> out;
        for (size_t i = 0; i < P.size(); ++i)
            if (prim_type(P[i]) & mask) out.push_back((int)i);
        return out;
    }
};

// Splits [0, nx) into contiguous ranges, one per thread (the x-slab split of
// Operator_Multithread); f(x0, x1, thread) runs once per range.
template <class F>
void parallel_x(uint32_t nx, int threads, F&& f) {
    int T = std::max(1, std::min<int>(threads, (int)nx));
    if (T == 1) {
        f(0u, nx, 0);
        return;
    }
    std::vector<std::thread> th;
    uint32_t per = nx / T, rem = nx % T, x0 = 0;
    for (int t = 0; t < T; ++t) {
        uint32_t cnt = per + ((uint32_t)t < rem ? 1 : 0);
        th.emplace_back([&f, x0, cnt, t] { f(x0, x0 + cnt, t); });
        x0 += cnt;
    }
    for (auto& t : th) t.join();
}

struct UpmlSlabO {
    int BC[6];
    uint32_t Size[6];
    uint32_t start[3], nl[3];
    std::vector<float> vv, vvfo, vvfn, ii, iifo, iifn;
    size_t at(int n, const uint32_t* l) const {
        return (((size_t)n * nl[0] + l[0]) * nl[1] + l[1]) * nl[2] + l[2];
    }
};

struct MurO {
    int ny, nyP, nyPP;
    bool top;
    uint32_t line, shift;
    uint32_t nl[2];
    double vph;
    std::vector<float> cp, cpp;
    uint32_t start_ts = 0;
};

struct AdeO {
    uint32_t count = 0;
    std::vector<uint32_t> pos[3];
    bool volt_on = false, curr_on = false, volt_lor_on = false, curr_lor_on = false;
    std::vector<float> v_int, v_ext, v_lor, i_int, i_ext, i_lor;  // [3][count]
};

}  // namespace

// The custom excitation's function of t, evaluated the way the function
// parser openEMS calls does arithmetic (excitation.cpp:233-271): tokens to
// postfix by operator precedence (shunting yard: ^ right-associative above
// unary minus, then * / %, then + -), then a stack machine in double.
struct OracleFunction {
    struct Tok {
        int kind;  // 0 number, 1 t, 2 operator, 3 function, 4 '(', 5 ')', 6 ','
        double v;
        char op;        // + - * / % ^ and 'u' for unary minus
        std::string fn;
    };
    std::vector<Tok> rpn;
    std::string err;

    static int prec(char op) { return op == '^' ? 4 : op == 'u' ? 3 : (op == '*' || op == '/' || op == '%') ? 2 : 1; }
    static bool right(char op) { return op == '^' || op == 'u'; }
    static int arity(const std::string& f) {
        static const char* two[] = {"atan2", "hypot", "max", "min", "pow"};
        for (const char* n : two)
            if (f == n) return 2;
        return 1;
    }

    bool parse(const std::string& s) {
        std::vector<Tok> toks;
        size_t i = 0;
        bool expect_operand = true;
        while (i < s.size()) {
            const char c = s[i];
            if (c == ' ' || c == '\t') { ++i; continue; }
            if ((c >= '0' && c <= '9') || c == '.') {
                char* end = nullptr;
                const double v = std::strtod(s.c_str() + i, &end);
                i = (size_t)(end - s.c_str());
                toks.push_back(Tok{0, v, 0, ""});
                expect_operand = false;
            } else if ((c >= 'a' && c <= 'z') || (c >= 'A' && c <= 'Z') || c == '_') {
                size_t e = i;
                while (e < s.size() && (std::isalnum((unsigned char)s[e]) || s[e] == '_')) ++e;
                const std::string id = s.substr(i, e - i);
                i = e;
                if (id == "t") toks.push_back(Tok{1, 0, 0, ""});
                else if (id == "pi") toks.push_back(Tok{0, 3.14159265358979323846, 0, ""});
                else if (id == "e") toks.push_back(Tok{0, 2.71828182845904523536, 0, ""});
                else { toks.push_back(Tok{3, 0, 0, id}); expect_operand = true; continue; }
                expect_operand = false;
            } else if (c == '(') { toks.push_back(Tok{4, 0, 0, ""}); ++i; expect_operand = true; }
            else if (c == ')') { toks.push_back(Tok{5, 0, 0, ""}); ++i; expect_operand = false; }
            else if (c == ',') { toks.push_back(Tok{6, 0, 0, ""}); ++i; expect_operand = true; }
            else if (std::strchr("+-*/%^", c)) {
                toks.push_back(Tok{2, 0, (c == '-' && expect_operand) ? 'u' : c, ""});
                ++i;
                expect_operand = true;
            } else { err = std::string("unsupported character ") + c; return false; }
        }
        std::vector<Tok> ops;
        for (const Tok& t : toks) {
            if (t.kind <= 1) rpn.push_back(t);
            else if (t.kind == 3) ops.push_back(t);
            else if (t.kind == 2) {
                if (t.op != 'u')
                    while (!ops.empty() && ops.back().kind == 2 &&
                           (prec(ops.back().op) > prec(t.op) || (prec(ops.back().op) == prec(t.op) && !right(t.op)))) {
                        rpn.push_back(ops.back());
                        ops.pop_back();
                    }
                ops.push_back(t);
            } else if (t.kind == 4) ops.push_back(t);
            else if (t.kind == 6 || t.kind == 5) {
                while (!ops.empty() && ops.back().kind != 4) { rpn.push_back(ops.back()); ops.pop_back(); }
                if (ops.empty()) { err = "unbalanced parentheses"; return false; }
                if (t.kind == 5) {
                    ops.pop_back();
                    if (!ops.empty() && ops.back().kind == 3) { rpn.push_back(ops.back()); ops.pop_back(); }
                }
            }
        }
        while (!ops.empty()) {
            if (ops.back().kind == 4) { err = "unbalanced parentheses"; return false; }
            rpn.push_back(ops.back());
            ops.pop_back();
        }
        return true;
    }

    double eval(double t) const {
        std::vector<double> st;
        for (const Tok& k : rpn) {
            if (k.kind == 0) { st.push_back(k.v); continue; }
            if (k.kind == 1) { st.push_back(t); continue; }
            if (k.kind == 2 && k.op == 'u') { st.back() = -st.back(); continue; }
            if (k.kind == 2) {
                const double b = st.back(); st.pop_back();
                double& a = st.back();
                switch (k.op) {
                    case '+': a = a + b; break;
                    case '-': a = a - b; break;
                    case '*': a = a * b; break;
                    case '/': a = a / b; break;
                    case '%': a = std::fmod(a, b); break;
                    default: a = std::pow(a, b); break;
                }
                continue;
            }
            const std::string& f = k.fn;
            if (arity(f) == 2) {
                const double b = st.back(); st.pop_back();
                double& a = st.back();
                if (f == "atan2") a = std::atan2(a, b);
                else if (f == "hypot") a = std::hypot(a, b);
                else if (f == "max") a = a > b ? a : b;
                else if (f == "min") a = a < b ? a : b;
                else a = std::pow(a, b);
                continue;
            }
            double& x = st.back();
            if (f == "abs") x = std::fabs(x);
            else if (f == "acos") x = std::acos(x);
            else if (f == "acosh") x = std::acosh(x);
            else if (f == "asin") x = std::asin(x);
            else if (f == "asinh") x = std::asinh(x);
            else if (f == "atan") x = std::atan(x);
            else if (f == "atanh") x = std::atanh(x);
            else if (f == "cbrt") x = std::cbrt(x);
            else if (f == "ceil") x = std::ceil(x);
            else if (f == "cos") x = std::cos(x);
            else if (f == "cosh") x = std::cosh(x);
            else if (f == "exp") x = std::exp(x);
            else if (f == "exp2") x = std::exp2(x);
            else if (f == "floor") x = std::floor(x);
            else if (f == "int") x = std::floor(x + 0.5);
            else if (f == "log") x = std::log(x);
            else if (f == "log10") x = std::log10(x);
            else if (f == "log2") x = std::log2(x);
            else if (f == "sin") x = std::sin(x);
            else if (f == "sinh") x = std::sinh(x);
            else if (f == "sqrt") x = std::sqrt(x);
            else if (f == "tan") x = std::tan(x);
            else if (f == "tanh") x = std::tanh(x);
            else x = std::trunc(x);
        }
        return st.empty() ? 0.0 : st.back();
    }
};

struct oracle_operator_s {
    uint32_t N[3];
    size_t NN;
    std::vector<double> lines[3];
    double unit;
    double bg[4];  // eps, kappa, mue, sigma (GetMaterial types 0..3)
    int BC[6];
    uint32_t pml[6];
    double mur_vph[6];
    double f0, fc;
    int excite_type = 0;
    double signal_period = 0;  // Excitation::m_SignalPeriod
    std::string function;      // the custom signal
    uint32_t nr_ts, oversampling;
    int threads;
    Csx csx;

    double dT = 0;
    std::vector<float> EC_C, EC_G, EC_L, EC_R;  // [3][x][y][z]
    std::vector<float> vv, vi, ii, iv;
    // Operator_Ext_Excitation lists
    std::vector<uint32_t> v_idx[3], c_idx[3];
    std::vector<uint16_t> v_dir, c_dir;
    std::vector<float> v_amp, c_amp;
    std::vector<uint32_t> v_delay, c_delay;
    std::vector<float> sig_v, sig_c;
    uint32_t length = 0, nyquist = 0, max_exc_ts = 0, probe_interval = 1, period_ts = 0;
    std::vector<MurO> mur;
    std::vector<UpmlSlabO> upml;
    std::vector<AdeO> ade;
    // lumped RLC
    std::vector<uint32_t> r_pos[3];
    std::vector<int> r_dir;
    std::vector<float> r_ilv, r_i2v, r_vv2, r_vj1, r_vj2, r_vvd, r_ib0, r_b1, r_b2;
    std::vector<fdtd_probe_desc> probes;
    // descriptor scratch
    std::vector<fdtd_upml_desc> upml_desc;
    std::vector<fdtd_ade_desc> ade_desc;
    std::vector<fdtd_mur_desc> mur_desc;
    fdtd_rlc_desc rlc_desc{};

    size_t at(int n, uint32_t x, uint32_t y, uint32_t z) const {
        return (size_t)n * NN + ((size_t)x * N[1] + y) * N[2] + z;
    }
    size_t at(int n, const uint32_t* p) const { return at(n, p[0], p[1], p[2]); }

    // ------------------------------------------------ mesh (operator.cpp:136-242)
    double GetDiscLine(int n, uint32_t pos, bool dual = false) const {
        if (n < 0 || n > 2) return 0.0;
        if (pos >= N[n]) return 0.0;
        if (!dual) return lines[n][pos];
        if (pos < N[n] - 1) return 0.5 * (lines[n][pos] + lines[n][pos + 1]);
        return lines[n][pos] + 0.5 * (lines[n][pos] - lines[n][pos - 1]);
    }
    double GetDiscDelta(int n, uint32_t pos, bool dual = false) const {
        if (n < 0 || n > 2) return 0.0;
        if (pos >= N[n]) return 0.0;
        if (!dual) {
            if (pos < N[n] - 1) return GetDiscLine(n, pos + 1, false) - GetDiscLine(n, pos, false);
            return GetDiscLine(n, pos, false) - GetDiscLine(n, pos - 1, false);
        }
        if (pos > 0) return GetDiscLine(n, pos, true) - GetDiscLine(n, pos - 1, true);
        return GetDiscLine(n, 1, false) - GetDiscLine(n, 0, false);
    }
    double GetEdgeLength(int n, const uint32_t* pos, bool dual = false) const {
        return GetDiscDelta(n, pos[n], dual) * unit;
    }
    double GetNodeWidth(int ny, const uint32_t* pos, bool dual = false) const {
        return GetEdgeLength(ny, pos, !dual);
    }
    double GetNodeWidth(int ny, const int* pos, bool dual = false) const {
        if (pos[0] < 0 || pos[1] < 0 || pos[2] < 0) return 0.0;
        uint32_t u[3] = {(uint32_t)pos[0], (uint32_t)pos[1], (uint32_t)pos[2]};
        return GetNodeWidth(ny, u, dual);
    }
    double GetNodeArea(int ny, const uint32_t* pos, bool dual = false) const {
        int nyP = (ny + 1) % 3, nyPP = (ny + 2) % 3;
        return GetNodeWidth(nyP, pos, dual) * GetNodeWidth(nyPP, pos, dual);
    }
    double GetNodeArea(int ny, const int* pos, bool dual = false) const {
        if (pos[0] < 0 || pos[1] < 0 || pos[2] < 0) return 0.0;
        uint32_t u[3] = {(uint32_t)pos[0], (uint32_t)pos[1], (uint32_t)pos[2]};
        return GetNodeArea(ny, u, dual);
    }
    double GetEdgeArea(int ny, const uint32_t* pos, bool dual = false) const { return GetNodeArea(ny, pos, dual); }
    bool GetYeeCoords(int ny, const uint32_t* pos, double* c, bool dual) const {
        for (int n = 0; n < 3; ++n) c[n] = GetDiscLine(n, pos[n], dual);
        c[ny] = GetDiscLine(ny, pos[ny], !dual);
        if (!dual) {
            if (pos[ny] >= N[ny] - 1) return false;
        } else {
            int nP = (ny + 1) % 3, nPP = (ny + 2) % 3;
            if ((pos[nP] >= N[nP] - 1) || (pos[nPP] >= N[nPP] - 1)) return false;
        }
        return true;
    }
    double GetRawDiscDelta(int ny, int pos) const {
        if (pos < 0) return lines[ny][0] - lines[ny][1];
        if (pos >= (int)N[ny] - 1) return lines[ny][N[ny] - 2] - lines[ny][N[ny] - 1];
        return lines[ny][pos + 1] - lines[ny][pos];
    }

    // ------------------------------------------- snapping (operator.cpp:244-345)
    uint32_t SnapToMeshLine(int ny, double coord, bool& inside, bool dual) const {
        inside = false;
        if (ny < 0 || ny > 2) return 0;
        if (coord < GetDiscLine(ny, 0)) return 0;
        uint32_t nl = N[ny];
        if (coord > GetDiscLine(ny, nl - 1)) return nl - 1;
        inside = true;
        if (!dual) {
            for (uint32_t n = 0; n < nl; ++n)
                if (coord <= GetDiscLine(ny, n, true)) return n;
        } else {
            for (uint32_t n = 1; n < nl; ++n)
                if (coord <= GetDiscLine(ny, n, false)) return n - 1;
        }
        return 0;
    }
    bool SnapToMesh(const double* c, uint32_t* ui, bool dual, bool* inside) const {
        bool ok = true;
        for (int n = 0; n < 3; ++n) {
            bool in = false;
            ui[n] = SnapToMeshLine(n, c[n], in, dual);
            ok &= in;
            if (inside) inside[n] = in;
        }
        return ok;
    }
    int SnapBox2Mesh(const double* start, const double* stop, uint32_t* uiStart, uint32_t* uiStop, bool dual,
                     int method, bool* bStartIn = nullptr, bool* bStopIn = nullptr) const {
        double l_start[3], l_stop[3];
        for (int n = 0; n < 3; ++n) {
            l_start[n] = std::fmin(start[n], stop[n]);
            l_stop[n] = std::fmax(start[n], stop[n]);
            double mn = GetDiscLine(n, 0), mx = GetDiscLine(n, N[n] - 1);
            if (((l_start[n] < mn) && (l_stop[n] < mn)) || ((l_start[n] > mx) && (l_stop[n] > mx))) return -2;
        }
        SnapToMesh(l_start, uiStart, dual, bStartIn);
        SnapToMesh(l_stop, uiStop, dual, bStopIn);
        int iDim = 0;
        if (method == 0) {
            for (int n = 0; n < 3; ++n)
                if (uiStop[n] > uiStart[n]) ++iDim;
            return iDim;
        }
        if (method == 1) {
            for (int n = 0; n < 3; ++n) {
                if (uiStop[n] > uiStart[n]) {
                    if ((GetDiscLine(n, uiStart[n], dual) > l_start[n]) && (uiStart[n] > 0)) --uiStart[n];
                    if ((GetDiscLine(n, uiStop[n], dual) < l_stop[n]) && (uiStop[n] < N[n] - 1)) ++uiStop[n];
                }
                if (uiStop[n] > uiStart[n]) ++iDim;
            }
            return iDim;
        }
        return -1;
    }

    // Operator::GetPrimitivesBoundBox (operator.cpp:1760-1778)
    std::vector<int> PrimitivesBoundBox(int px, int py, int pz, int mask) const {
        double bb[6];
        int p[3] = {px, py, pz};
        for (int n = 0; n < 3; ++n) {
            if (p[n] < 0) {
                bb[2 * n] = GetDiscLine(n, 0);
                bb[2 * n + 1] = GetDiscLine(n, N[n] - 1);
            } else {
                bb[2 * n] = GetDiscLine(n, (uint32_t)std::max(0, p[n] - 1));
                bb[2 * n + 1] = GetDiscLine(n, (uint32_t)std::min((int)N[n] - 1, p[n] + 1));
            }
        }
        return csx.by_bound_box(bb, mask);
    }

    // Operator::GetMaterial (operator.cpp:1251-1298): 0 eps_r, 1 kappa, 2 mue_r, 3 sigma
    double GetMaterial(const double* c, int type, const std::vector<int>& vPrims) const {
        int w = csx.by_coord_priority(c, vPrims);
        if (w >= 0 && csx.P[w].kind == 1) {
            const oracle_prim& m = csx.P[w];
            switch (type) {
                case 0: return m.eps;
                case 1: return m.kappa;
                case 2: return m.mue;
                case 3: return m.sigma;
            }
            return 0;
        }
        return bg[type];
    }

    // Operator::AverageMatQuarterCell (operator.cpp:1406-1518)
    void AverageMatQuarterCell(int ny, const uint32_t* pos, double* EffMat, const std::vector<int>& vPrims) const {
        int n = ny;
        double coord[3], shiftCoord[3];
        int nP = (n + 1) % 3, nPP = (n + 2) % 3;
        coord[0] = lines[0][pos[0]];
        coord[1] = lines[1][pos[1]];
        coord[2] = lines[2][pos[2]];
        double delta = GetRawDiscDelta(n, (int)pos[n]);
        double deltaP = GetRawDiscDelta(nP, (int)pos[nP]);
        double deltaPP = GetRawDiscDelta(nPP, (int)pos[nPP]);
        double delta_M = GetRawDiscDelta(n, (int)pos[n] - 1);
        double deltaP_M = GetRawDiscDelta(nP, (int)pos[nP] - 1);
        double deltaPP_M = GetRawDiscDelta(nPP, (int)pos[nPP] - 1);
        int loc_pos[3] = {(int)pos[0], (int)pos[1], (int)pos[2]};
        double A_n, area = 0;

        // epsilon, kappa: four quarter cells around the edge
        shiftCoord[n] = coord[n] + delta * 0.5;
        shiftCoord[nP] = coord[nP] + deltaP * 0.25;
        shiftCoord[nPP] = coord[nPP] + deltaPP * 0.25;
        A_n = GetNodeArea(ny, loc_pos, true);
        EffMat[0] = GetMaterial(shiftCoord, 0, vPrims) * A_n;
        EffMat[1] = GetMaterial(shiftCoord, 1, vPrims) * A_n;
        area += A_n;

        shiftCoord[n] = coord[n] + delta * 0.5;
        shiftCoord[nP] = coord[nP] - deltaP_M * 0.25;
        shiftCoord[nPP] = coord[nPP] + deltaPP * 0.25;
        --loc_pos[nP];
        A_n = GetNodeArea(ny, loc_pos, true);
        EffMat[0] += GetMaterial(shiftCoord, 0, vPrims) * A_n;
        EffMat[1] += GetMaterial(shiftCoord, 1, vPrims) * A_n;
        area += A_n;

        shiftCoord[n] = coord[n] + delta * 0.5;
        shiftCoord[nP] = coord[nP] + deltaP * 0.25;
        shiftCoord[nPP] = coord[nPP] - deltaPP_M * 0.25;
        ++loc_pos[nP];
        --loc_pos[nPP];
        A_n = GetNodeArea(ny, loc_pos, true);
        EffMat[0] += GetMaterial(shiftCoord, 0, vPrims) * A_n;
        EffMat[1] += GetMaterial(shiftCoord, 1, vPrims) * A_n;
        area += A_n;

        shiftCoord[n] = coord[n] + delta * 0.5;
        shiftCoord[nP] = coord[nP] - deltaP_M * 0.25;
        shiftCoord[nPP] = coord[nPP] - deltaPP_M * 0.25;
        --loc_pos[nP];
        A_n = GetNodeArea(ny, loc_pos, true);
        EffMat[0] += GetMaterial(shiftCoord, 0, vPrims) * A_n;
        EffMat[1] += GetMaterial(shiftCoord, 1, vPrims) * A_n;
        area += A_n;

        EffMat[0] *= kEps0 / area;
        EffMat[1] /= area;

        // mue, sigma: the two half cells along the edge's dual line
        loc_pos[0] = (int)pos[0];
        loc_pos[1] = (int)pos[1];
        loc_pos[2] = (int)pos[2];
        double length = 0;
        shiftCoord[n] = coord[n] - delta_M * 0.25;
        shiftCoord[nP] = coord[nP] + deltaP * 0.5;
        shiftCoord[nPP] = coord[nPP] + deltaPP * 0.5;
        --loc_pos[n];
        double delta_ny = GetNodeWidth(n, loc_pos, true);
        EffMat[2] = delta_ny / GetMaterial(shiftCoord, 2, vPrims);
        double sigma = GetMaterial(shiftCoord, 3, vPrims);
        if (sigma)
            EffMat[3] = delta_ny / sigma;
        else
            EffMat[3] = 0;
        length = delta_ny;

        shiftCoord[n] = coord[n] + delta * 0.25;
        shiftCoord[nP] = coord[nP] + deltaP * 0.5;
        shiftCoord[nPP] = coord[nPP] + deltaPP * 0.5;
        ++loc_pos[n];
        delta_ny = GetNodeWidth(n, loc_pos, true);
        EffMat[2] += delta_ny / GetMaterial(shiftCoord, 2, vPrims);
        sigma = GetMaterial(shiftCoord, 3, vPrims);
        if (sigma)
            EffMat[3] += delta_ny / sigma;
        else
            EffMat[3] = 0;
        length += delta_ny;

        EffMat[2] = length * kMue0 / EffMat[2];
        if (EffMat[3]) EffMat[3] = length / EffMat[3];
    }

    // Operator::Calc_ECPos (operator.cpp:1176-1224)
    void Calc_ECPos(int ny, const uint32_t* pos, double* EC, const std::vector<int>& vPrims) const {
        double EffMat[4];
        AverageMatQuarterCell(ny, pos, EffMat, vPrims);
        double delta = GetEdgeLength(ny, pos);
        double area = GetEdgeArea(ny, pos);
        if (delta) {
            EC[0] = EffMat[0] * area / delta;
            EC[1] = EffMat[1] * area / delta;
        } else {
            EC[0] = 0;
            EC[1] = 0;
        }
        delta = GetEdgeLength(ny, pos, true);
        area = GetEdgeArea(ny, pos, true);
        if (delta) {
            EC[2] = EffMat[2] * area / delta;
            EC[3] = EffMat[3] * area / delta;
        } else {
            EC[2] = 0;
            EC[3] = 0;
        }
    }

    // Operator::Calc_EC_Range over all x (operator.cpp:1780-1803), x planes
    // split over threads as Operator_Multithread does
    void Calc_EC() {
        EC_C.assign(3 * NN, 0.f);
        EC_G.assign(3 * NN, 0.f);
        EC_L.assign(3 * NN, 0.f);
        EC_R.assign(3 * NN, 0.f);
        parallel_x(N[0], threads, [&](uint32_t x0, uint32_t x1, int) {
            uint32_t pos[3];
            double inEC[4];
            for (pos[0] = x0; pos[0] < x1; ++pos[0])
                for (pos[1] = 0; pos[1] < N[1]; ++pos[1]) {
                    std::vector<int> vPrims = PrimitivesBoundBox((int)pos[0], (int)pos[1], -1, T_MATERIAL);
                    for (pos[2] = 0; pos[2] < N[2]; ++pos[2])
                        for (int n = 0; n < 3; ++n) {
                            Calc_ECPos(n, pos, inEC, vPrims);
                            size_t i = at(n, pos);
                            EC_C[i] = (float)inEC[0];
                            EC_G[i] = (float)inEC[1];
                            EC_L[i] = (float)inEC[2];
                            EC_R[i] = (float)inEC[3];
                        }
                }
        });
    }

    // AdrOp::GetPos with SetReflection2Cell: each axis' shifted index is
    // mirrored back onto the grid (tools/AdrOp.cpp:197-202, offset 1)
    size_t shifted(int n, const uint32_t* pos, int s0, int s1, int s2) const {
        int s[3] = {s0, s1, s2};
        uint32_t q[3];
        for (int a = 0; a < 3; ++a) {
            int rel = s[a];
            int p = (int)pos[a];
            if (rel + p < 0) rel = -2 * p - rel - 1;
            if (rel + p > (int)N[a] - 1) rel = 2 * ((int)N[a] - 1 - p) - rel + 1;
            q[a] = (uint32_t)(p + rel);
        }
        return at(n, q);
    }

    static double min4(const double* v) {
        double m = v[0];
        for (int k = 1; k < 4; ++k)
            if (v[k] < m) m = v[k];
        return m;
    }

    // Operator::CalcTimestep_Var3 (operator.cpp:1897-1971).  The AdrOp shift
    // state is followed literally: Shift(nP,-1) then Shift(nPP,-1) leaves both
    // shifts set, and GetShiftedPos adds to the current shift.
    double CalcTimestep_Var3() const {
        std::vector<double> best(std::max(1, threads), 1e200);
        parallel_x(N[0], threads, [&](uint32_t x0, uint32_t x1, int t) {
            double dTl = 1e200;
            uint32_t pos[3];
            for (int n = 0; n < 3; ++n) {
                int nP = (n + 1) % 3, nPP = (n + 2) % 3;
                for (pos[0] = x0; pos[0] < x1; ++pos[0])
                    for (pos[1] = 0; pos[1] < N[1]; ++pos[1])
                        for (pos[2] = 0; pos[2] < N[2]; ++pos[2]) {
                            int sh[3] = {0, 0, 0};
                            auto S = [&](int axis, int step, int axis2 = -1, int step2 = 0) {
                                int s[3] = {sh[0], sh[1], sh[2]};
                                if (axis >= 0) s[axis] += step;
                                if (axis2 >= 0) s[axis2] += step2;
                                return shifted(0, pos, s[0], s[1], s[2]);
                            };
                            const float* L = EC_L.data();
                            const float* C = EC_C.data();
                            const size_t cn = (size_t)n * NN, cP = (size_t)nP * NN, cPP = (size_t)nPP * NN;
                            size_t ipos = S(-1, 0);
                            double wqp = 1 / (L[cPP + ipos] * C[cn + S(nP, 1)]) + 1 / (L[cPP + ipos] * C[cn + ipos]);
                            wqp += 1 / (L[cP + ipos] * C[cn + S(nPP, 1)]) + 1 / (L[cP + ipos] * C[cn + ipos]);
                            sh[nP] = -1;
                            ipos = S(-1, 0);
                            wqp += 1 / (L[cPP + ipos] * C[cn + S(nP, 1)]) + 1 / (L[cPP + ipos] * C[cn + ipos]);
                            sh[nPP] = -1;
                            ipos = S(-1, 0);
                            wqp += 1 / (L[cP + ipos] * C[cn + S(nPP, 1)]) + 1 / (L[cP + ipos] * C[cn + ipos]);

                            sh[0] = sh[1] = sh[2] = 0;
                            ipos = S(-1, 0);
                            double wt_4[4];
                            wt_4[0] = 1 / (L[cPP + ipos] * C[cP + ipos]);
                            wt_4[1] = 1 / (L[cPP + S(nP, -1)] * C[cP + ipos]);
                            wt_4[2] = 1 / (L[cP + ipos] * C[cPP + ipos]);
                            wt_4[3] = 1 / (L[cP + S(nPP, -1)] * C[cPP + ipos]);
                            double wt1 = wt_4[0] + wt_4[1] + wt_4[2] + wt_4[3] - 2 * min4(wt_4);

                            wt_4[0] = 1 / (L[cPP + ipos] * C[cP + S(n, 1)]);
                            wt_4[1] = 1 / (L[cPP + S(nP, -1)] * C[cP + S(n, 1)]);
                            wt_4[2] = 1 / (L[cP + ipos] * C[cPP + S(n, 1)]);
                            wt_4[3] = 1 / (L[cP + S(nPP, -1)] * C[cPP + S(n, 1)]);
                            double wt2 = wt_4[0] + wt_4[1] + wt_4[2] + wt_4[3] - 2 * min4(wt_4);

                            double w_total = wqp + wt1 + wt2;
                            double newT = 2 / std::sqrt(w_total);
                            if ((newT < dTl) && (newT > 0.0)) dTl = newT;
                        }
            }
            best[(size_t)t] = dTl;  // the minimum does not depend on the visiting order
        });
        double d = 1e200;
        for (double b : best) d = std::min(d, b);
        return d;
    }

    // Operator::Calc_ECOperatorPos (operator.cpp:943-971)
    void Calc_ECOperatorPos(int n, const uint32_t* pos) {
        size_t i = at(n, pos);
        double C = EC_C[i];
        double G = EC_G[i];
        if (C > 0) {
            vv[i] = (float)((1.0 - dT * G / 2.0 / C) / (1.0 + dT * G / 2.0 / C));
            vi[i] = (float)((dT / C) / (1.0 + dT * G / 2.0 / C));
        } else {
            vv[i] = 0;
            vi[i] = 0;
        }
        double L = EC_L[i];
        double R = EC_R[i];
        if (L > 0) {
            ii[i] = (float)((1.0 - dT * R / 2.0 / L) / (1.0 + dT * R / 2.0 / L));
            iv[i] = (float)((dT / L) / (1.0 + dT * R / 2.0 / L));
        } else {
            ii[i] = 0;
            iv[i] = 0;
        }
    }
    void SetVV(int n, const uint32_t* p, float v) { vv[at(n, p)] = v; }
    void SetVI(int n, const uint32_t* p, float v) { vi[at(n, p)] = v; }
    void SetII(int n, const uint32_t* p, float v) { ii[at(n, p)] = v; }
    void SetIV(int n, const uint32_t* p, float v) { iv[at(n, p)] = v; }

    // Operator::ApplyElectricBC (operator.cpp:1086-1125)
    void ApplyElectricBC(const bool* dirs) {
        uint32_t pos[3];
        for (int n = 0; n < 3; ++n) {
            int nP = (n + 1) % 3, nPP = (n + 2) % 3;
            for (pos[nP] = 0; pos[nP] < N[nP]; ++pos[nP])
                for (pos[nPP] = 0; pos[nPP] < N[nPP]; ++pos[nPP]) {
                    if (dirs[2 * n]) {
                        pos[n] = 0;
                        SetVV(nP, pos, 0); SetVI(nP, pos, 0);
                        SetVV(nPP, pos, 0); SetVI(nPP, pos, 0);
                    }
                    if (dirs[2 * n + 1]) {
                        pos[n] = N[n] - 1;
                        SetVV(n, pos, 0); SetVI(n, pos, 0);
                        SetVV(nP, pos, 0); SetVI(nP, pos, 0);
                        SetVV(nPP, pos, 0); SetVI(nPP, pos, 0);
                    }
                }
        }
    }

    // Operator::ApplyMagneticBC (operator.cpp:1127-1174)
    void ApplyMagneticBC(const bool* dirs) {
        uint32_t pos[3];
        for (int n = 0; n < 3; ++n) {
            int nP = (n + 1) % 3, nPP = (n + 2) % 3;
            for (pos[nP] = 0; pos[nP] < N[nP]; ++pos[nP])
                for (pos[nPP] = 0; pos[nPP] < N[nPP]; ++pos[nPP]) {
                    if (dirs[2 * n]) {
                        pos[n] = 0;
                        SetII(n, pos, 0); SetIV(n, pos, 0);
                        SetII(nP, pos, 0); SetIV(nP, pos, 0);
                        SetII(nPP, pos, 0); SetIV(nPP, pos, 0);
                    }
                    if (dirs[2 * n + 1]) {
                        pos[n] = N[n] - 2;
                        SetII(nP, pos, 0); SetIV(nP, pos, 0);
                        SetII(nPP, pos, 0); SetIV(nPP, pos, 0);
                    }
                    pos[n] = N[n] - 1;
                    SetII(n, pos, 0); SetIV(n, pos, 0);
                    SetII(nP, pos, 0); SetIV(nP, pos, 0);
                    SetII(nPP, pos, 0); SetIV(nPP, pos, 0);
                }
        }
    }

    // Operator::CalcPEC_Range (operator.cpp:1986-2020)
    void CalcPEC() {
        parallel_x(N[0], threads, [&](uint32_t x0, uint32_t x1, int) {
            double coord[3];
            uint32_t pos[3];
            for (pos[0] = x0; pos[0] < x1; ++pos[0])
                for (pos[1] = 0; pos[1] < N[1]; ++pos[1]) {
                    std::vector<int> vPrims = PrimitivesBoundBox((int)pos[0], (int)pos[1], -1, T_MATERIAL | T_METAL);
                    for (pos[2] = 0; pos[2] < N[2]; ++pos[2])
                        for (int n = 0; n < 3; ++n) {
                            GetYeeCoords(n, pos, coord, false);
                            int w = csx.by_coord_priority(coord, vPrims);
                            if (w >= 0 && csx.P[w].kind == 2) {
                                SetVV(n, pos, 0);
                                SetVI(n, pos, 0);
                            }
                        }
                }
        });
    }

    // Operator::Calc_LumpedElements (operator.cpp:1535-1712)
    void Calc_LumpedElements() {
        for (int k : csx.by_type(T_LUMPED)) {
            const oracle_prim& P = csx.P[k];
            double C = P.C;
            if (C <= 0) C = NAN;
            double R = P.R;
            if (R < 0) R = NAN;
            // IsLEparRC (operator.cpp:1714-1724)
            if (!((P.le_type == FDTD_LE_PARALLEL) && !(P.L > 0.0))) continue;
            if (std::isnan(R) && std::isnan(C)) continue;
            int ny = P.ny;
            if (ny < 0 || ny > 2) continue;
            int nyP = (ny + 1) % 3, nyPP = (ny + 2) % 3;
            uint32_t uiStart[3], uiStop[3];
            int dim = SnapBox2Mesh(P.start, P.stop, uiStart, uiStop, false, 0);
            if (dim <= 0) continue;
            if (uiStart[ny] == uiStop[ny]) continue;
            uint32_t pos[3];
            double unitGC = 0;
            for (pos[ny] = uiStart[ny]; pos[ny] < uiStop[ny]; ++pos[ny]) {
                double unitGC_Plane = 0;
                for (pos[nyP] = uiStart[nyP]; pos[nyP] <= uiStop[nyP]; ++pos[nyP])
                    for (pos[nyPP] = uiStart[nyPP]; pos[nyPP] <= uiStop[nyPP]; ++pos[nyPP])
                        unitGC_Plane += GetEdgeArea(ny, pos) / GetEdgeLength(ny, pos);
                unitGC += 1 / unitGC_Plane;
            }
            unitGC = 1 / unitGC;
            bool caps = P.caps != 0;
            double kappa = 0, epsilon = 0;
            if (R > 0) kappa = 1 / R / unitGC;
            if (C > 0) {
                epsilon = C / unitGC;
                if (epsilon < kEps0) C = 0;
            }
            for (pos[ny] = uiStart[ny]; pos[ny] < uiStop[ny]; ++pos[ny])
                for (pos[nyP] = uiStart[nyP]; pos[nyP] <= uiStop[nyP]; ++pos[nyP])
                    for (pos[nyPP] = uiStart[nyPP]; pos[nyPP] <= uiStop[nyPP]; ++pos[nyPP]) {
                        size_t i = at(ny, pos);
                        if (C > 0) EC_C[i] = (float)(epsilon * GetEdgeArea(ny, pos) / GetEdgeLength(ny, pos));
                        if (R > 0) EC_G[i] = (float)(kappa * GetEdgeArea(ny, pos) / GetEdgeLength(ny, pos));
                        if (R == 0) {
                            SetVV(ny, pos, 0);
                            SetVI(ny, pos, 0);
                        } else {
                            Calc_ECOperatorPos(ny, pos);
                        }
                    }
            if (caps)
                for (pos[nyP] = uiStart[nyP]; pos[nyP] <= uiStop[nyP]; ++pos[nyP])
                    for (pos[nyPP] = uiStart[nyPP]; pos[nyPP] <= uiStop[nyPP]; ++pos[nyPP]) {
                        pos[ny] = uiStart[ny];
                        if (pos[nyP] < uiStop[nyP]) { SetVV(nyP, pos, 0); SetVI(nyP, pos, 0); }
                        if (pos[nyPP] < uiStop[nyPP]) { SetVV(nyPP, pos, 0); SetVI(nyPP, pos, 0); }
                        pos[ny] = uiStop[ny];
                        if (pos[nyP] < uiStop[nyP]) { SetVV(nyP, pos, 0); SetVI(nyP, pos, 0); }
                        if (pos[nyPP] < uiStop[nyPP]) { SetVV(nyPP, pos, 0); SetVI(nyPP, pos, 0); }
                    }
        }
    }

    // Operator_Ext_Excitation::BuildExtension (operator_ext_excitation.cpp:101-285);
    // excitation types 0/1 soft/hard E, 2/3 soft/hard H
    void BuildExcitation() {
        uint32_t pos[3];
        double vc[3], cc[3];
        for (pos[2] = 0; pos[2] < N[2]; ++pos[2])
            for (pos[1] = 0; pos[1] < N[1]; ++pos[1]) {
                std::vector<int> vPrims = PrimitivesBoundBox(-1, (int)pos[1], (int)pos[2], T_EXCITATION);
                for (pos[0] = 0; pos[0] < N[0]; ++pos[0]) {
                    for (int n = 0; n < 3; ++n) {
                        if (!GetYeeCoords(n, pos, vc, false)) continue;
                        int w = csx.by_coord_priority(vc, vPrims);
                        if (w < 0) continue;
                        const oracle_prim& e = csx.P[w];
                        if (e.exc_type == 0 || e.exc_type == 1) {
                            double amp = e.exc_vec[n] * GetEdgeLength(n, pos);
                            if (amp != 0) {
                                v_amp.push_back((float)amp);
                                v_delay.push_back((uint32_t)(e.delay / dT));
                                v_dir.push_back((uint16_t)n);
                                for (int a = 0; a < 3; ++a) v_idx[a].push_back(pos[a]);
                            }
                            if (e.exc_type == 1) {
                                SetVV(n, pos, 0);
                                SetVI(n, pos, 0);
                            }
                        }
                    }
                    for (int n = 0; n < 3; ++n) {
                        if ((pos[0] >= N[0] - 1) || (pos[1] >= N[1] - 1) || (pos[2] >= N[2] - 1)) continue;
                        if (!GetYeeCoords(n, pos, cc, true)) continue;
                        int w = csx.by_coord_priority(cc, vPrims);
                        if (w < 0) continue;
                        const oracle_prim& e = csx.P[w];
                        if (e.exc_type == 2 || e.exc_type == 3) {
                            double amp = e.exc_vec[n] * GetEdgeLength(n, pos, true);
                            if (amp != 0) {
                                c_amp.push_back((float)amp);
                                c_delay.push_back((uint32_t)(e.delay / dT));
                                c_dir.push_back((uint16_t)n);
                                for (int a = 0; a < 3; ++a) c_idx[a].push_back(pos[a]);
                            }
                            if (e.exc_type == 3) {
                                SetII(n, pos, 0);
                                SetIV(n, pos, 0);
                            }
                        }
                    }
                }
            }
    }

    // Operator_Ext_Mur_ABC::SetDirection + BuildExtension (operator_ext_mur_abc.cpp:88-195)
    void BuildMur(MurO& M) {
        uint32_t pos[3] = {0, 0, 0};
        pos[M.ny] = M.line;
        double delta = std::fabs(GetEdgeLength(M.ny, pos));
        double coord[3] = {GetDiscLine(0, pos[0]), GetDiscLine(1, pos[1]), GetDiscLine(2, pos[2])};
        if (M.line == 0)
            coord[M.ny] = GetDiscLine(M.ny, pos[M.ny]) + delta / 2 / unit;
        else
            coord[M.ny] = GetDiscLine(M.ny, pos[M.ny]) - delta / 2 / unit;
        int posBB[3];
        posBB[M.ny] = (int)pos[M.ny];
        posBB[M.nyPP] = -1;
        M.cp.assign((size_t)M.nl[0] * M.nl[1], 0.f);
        M.cpp.assign((size_t)M.nl[0] * M.nl[1], 0.f);
        for (pos[M.nyP] = 0; pos[M.nyP] < M.nl[0]; ++pos[M.nyP]) {
            posBB[M.nyP] = (int)pos[M.nyP];
            std::vector<int> vPrims = PrimitivesBoundBox(posBB[0], posBB[1], posBB[2], T_MATERIAL);
            coord[M.nyP] = GetDiscLine(M.nyP, pos[M.nyP]);
            for (pos[M.nyPP] = 0; pos[M.nyPP] < M.nl[1]; ++pos[M.nyPP]) {
                coord[M.nyPP] = GetDiscLine(M.nyPP, pos[M.nyPP]);
                int w = csx.by_coord_priority(coord, vPrims);
                size_t k = (size_t)pos[M.nyP] * M.nl[1] + pos[M.nyPP];
                double c0t;
                if (w >= 0) {
                    const oracle_prim& m = csx.P[w];
                    double eps = m.eps, mue = m.mue;
                    if (M.vph > 0.0)
                        c0t = M.vph * dT;
                    else
                        c0t = kC0 * dT / std::sqrt(eps * mue);
                    M.cp[k] = (float)((c0t - delta) / (c0t + delta));
                    if (M.vph > 0.0)
                        c0t = M.vph * dT;
                    else
                        c0t = kC0 * dT / std::sqrt(eps * mue);
                    M.cpp[k] = (float)((c0t - delta) / (c0t + delta));
                } else {
                    if (M.vph > 0.0)
                        c0t = M.vph * dT;
                    else
                        c0t = kC0 / std::sqrt(bg[0] * bg[2]) * dT;
                    M.cp[k] = (float)((c0t - delta) / (c0t + delta));
                    M.cpp[k] = M.cp[k];
                }
            }
        }
    }

    // Operator_Ext_UPML::Create_UPML (operator_ext_upml.cpp:77-201), Cartesian part
    // false when a slab's range leaves the grid: the reference computes the
    // ranges in unsigned arithmetic, so the y / z slabs of a grid with fewer
    // than size[0]+2 x-lines (size[0] = 8 when x-min is not PML) wrap around
    bool CreateUPML() {
        int BC[6];
        uint32_t size[6];
        for (int k = 0; k < 6; ++k) {
            BC[k] = this->BC[k];
            size[k] = pml[k];
        }
        for (int n = 0; n < 3; ++n)
            if ((size[2 * n] * (BC[2 * n] == 3) + size[2 * n + 1] * (BC[2 * n + 1] == 3)) >= N[n]) {
                BC[2 * n] = 0; size[2 * n] = 0;
                BC[2 * n + 1] = 0; size[2 * n + 1] = 0;
            }
        uint32_t start[3] = {0, 0, 0};
        uint32_t stop[3] = {N[0] - 1, N[1] - 1, N[2] - 1};
        auto add = [&]() {
            UpmlSlabO s;
            for (int k = 0; k < 6; ++k) {
                s.BC[k] = BC[k];
                s.Size[k] = size[k];
            }
            for (int n = 0; n < 3; ++n) {
                s.start[n] = start[n];
                s.nl[n] = stop[n] - start[n] + 1;
            }
            upml.push_back(std::move(s));
        };
        if (BC[0] == 3) { start[0] = 0; stop[0] = size[0]; add(); }
        if (BC[1] == 3) { start[0] = N[0] - 1 - size[1]; stop[0] = N[0] - 1; add(); }
        start[0] = (size[0] + 1) * (BC[0] == 3);
        stop[0] = N[0] - 1 - (size[0] + 1) * (BC[1] == 3);
        if (BC[2] == 3) { start[1] = 0; stop[1] = size[2]; add(); }
        if (BC[3] == 3) { start[1] = N[1] - 1 - size[3]; stop[1] = N[1] - 1; add(); }
        start[1] = (size[2] + 1) * (BC[2] == 3);
        stop[1] = N[1] - 1 - (size[3] + 1) * (BC[3] == 3);
        if (BC[4] == 3) { start[2] = 0; stop[2] = size[4]; add(); }
        if (BC[5] == 3) { start[2] = N[2] - 1 - size[5]; stop[2] = N[2] - 1; add(); }
        for (const UpmlSlabO& s : upml)
            for (int n = 0; n < 3; ++n)
                if (s.nl[n] == 0 || (uint64_t)s.start[n] + s.nl[n] > N[n]) return false;
        return true;
    }

    // default grading function " -log(1e-6)*log(2.5)/(2*dl*Z*(pow(2.5,W/dl)-1)) * pow(2.5, D/dl) "
    // (operator_ext_upml.cpp:31) with vars D, dl, W, Z, N
    static double grading(const double* v) {
        double D = v[0], dl = v[1], W = v[2], Z = v[3];
        return -log(1e-6) * log(2.5) / (2 * dl * Z * (pow(2.5, W / dl) - 1)) * pow(2.5, D / dl);
    }

    // Operator_Ext_UPML::CalcGradingKappa (operator_ext_upml.cpp:289-363), Cartesian
    void CalcGradingKappa(const UpmlSlabO& u, int ny, const uint32_t* pos, double Zm, double* kappa_v,
                          double* kappa_i) const {
        double depth = 0, width = 0;
        for (int n = 0; n < 3; ++n) {
            if ((pos[n] <= u.Size[2 * n]) && (u.BC[2 * n] == 3)) {
                width = (GetDiscLine(n, u.Size[2 * n]) - GetDiscLine(n, 0)) * unit;
                depth = width - (GetDiscLine(n, pos[n]) - GetDiscLine(n, 0)) * unit;
                if (n == ny) depth -= GetEdgeLength(n, pos) / 2;
                double vars[5] = {depth, width / u.Size[2 * n], width, Zm, (double)u.Size[2 * n]};
                if (depth > 0)
                    kappa_v[n] = grading(vars);
                else
                    kappa_v[n] = 0;
                if (n == ny) depth += GetEdgeLength(n, pos) / 2;
                if (n != ny) depth -= GetEdgeLength(n, pos) / 2;
                if (depth < 0) depth = 0;
                vars[0] = depth;
                if (depth > 0)
                    kappa_i[n] = grading(vars);
                else
                    kappa_i[n] = 0;
            } else if ((pos[n] >= N[n] - 1 - u.Size[2 * n + 1]) && (u.BC[2 * n + 1] == 3)) {
                width = (GetDiscLine(n, N[n] - 1) - GetDiscLine(n, N[n] - u.Size[2 * n + 1] - 1)) * unit;
                depth = width - (GetDiscLine(n, N[n] - 1) - GetDiscLine(n, pos[n])) * unit;
                if (n == ny) depth += GetEdgeLength(n, pos) / 2;
                double vars[5] = {depth, width / (u.Size[2 * n]), width, Zm, (double)u.Size[2 * n]};
                if (depth > 0)
                    kappa_v[n] = grading(vars);
                else
                    kappa_v[n] = 0;
                if (n == ny) depth -= GetEdgeLength(n, pos) / 2;
                if (n != ny) depth += GetEdgeLength(n, pos) / 2;
                if (depth > width) depth = 0;
                vars[0] = depth;
                if (depth > 0)
                    kappa_i[n] = grading(vars);
                else
                    kappa_i[n] = 0;
            } else {
                kappa_v[n] = 0;
                kappa_i[n] = 0;
            }
        }
    }

    // Operator_Ext_UPML::BuildExtension (operator_ext_upml.cpp:365-466)
    void BuildUPML(UpmlSlabO& u) {
        size_t nloc = 3 * (size_t)u.nl[0] * u.nl[1] * u.nl[2];
        u.vv.assign(nloc, 0.f); u.vvfo.assign(nloc, 0.f); u.vvfn.assign(nloc, 0.f);
        u.ii.assign(nloc, 0.f); u.iifo.assign(nloc, 0.f); u.iifn.assign(nloc, 0.f);
        parallel_x(u.nl[0], threads, [&](uint32_t l0, uint32_t l1, int) {
            uint32_t pos[3], loc[3];
            double kappa_v[3] = {0, 0, 0}, kappa_i[3] = {0, 0, 0}, eff[4];
            for (loc[0] = l0; loc[0] < l1; ++loc[0]) {
                pos[0] = loc[0] + u.start[0];
                for (loc[1] = 0; loc[1] < u.nl[1]; ++loc[1]) {
                    pos[1] = loc[1] + u.start[1];
                    std::vector<int> vPrims = PrimitivesBoundBox((int)pos[0], (int)pos[1], -1, T_MATERIAL);
                    for (loc[2] = 0; loc[2] < u.nl[2]; ++loc[2]) {
                        pos[2] = loc[2] + u.start[2];
                        for (int n = 0; n < 3; ++n) {
                            AverageMatQuarterCell(n, pos, eff, vPrims);
                            CalcGradingKappa(u, n, pos, kZ0, kappa_v, kappa_i);
                            int nP = (n + 1) % 3, nPP = (n + 2) % 3;
                            size_t g = at(n, pos), l = u.at(n, loc);
                            if (((kappa_v[0] + kappa_v[1] + kappa_v[2]) != 0) && (eff[1] < 1e3)) {
                                if ((vv[g] + vi[g]) != 0) {
                                    vv[g] = (float)((2 * kEps0 - kappa_v[nP] * dT) / (2 * kEps0 + kappa_v[nP] * dT));
                                    vi[g] = (float)((2 * kEps0 * dT) / (2 * kEps0 + kappa_v[nP] * dT) *
                                                    GetEdgeLength(n, pos) / GetEdgeArea(n, pos));
                                    u.vv[l] = (float)((2 * kEps0 - kappa_v[nPP] * dT) / (2 * kEps0 + kappa_v[nPP] * dT));
                                    u.vvfn[l] = (float)((2 * kEps0 + kappa_v[n] * dT) /
                                                        (2 * kEps0 + kappa_v[nPP] * dT) / eff[0]);
                                    u.vvfo[l] = (float)((2 * kEps0 - kappa_v[n] * dT) /
                                                        (2 * kEps0 + kappa_v[nPP] * dT) / eff[0]);
                                }
                            } else {
                                u.vv[l] = vv[g];
                                vv[g] = 0;
                                u.vvfo[l] = 0;
                                u.vvfn[l] = 1;
                            }
                            if ((kappa_i[0] + kappa_i[1] + kappa_i[2]) != 0) {
                                if ((ii[g] + iv[g]) != 0) {
                                    ii[g] = (float)((2 * kEps0 - kappa_i[nP] * dT) / (2 * kEps0 + kappa_i[nP] * dT));
                                    iv[g] = (float)((2 * kEps0 * dT) / (2 * kEps0 + kappa_i[nP] * dT) *
                                                    GetEdgeLength(n, pos, true) / GetEdgeArea(n, pos, true));
                                    u.ii[l] = (float)((2 * kEps0 - kappa_i[nPP] * dT) / (2 * kEps0 + kappa_i[nPP] * dT));
                                    u.iifn[l] = (float)((2 * kEps0 + kappa_i[n] * dT) /
                                                        (2 * kEps0 + kappa_i[nPP] * dT) / eff[2]);
                                    u.iifo[l] = (float)((2 * kEps0 - kappa_i[n] * dT) /
                                                        (2 * kEps0 + kappa_i[nPP] * dT) / eff[2]);
                                }
                            } else {
                                u.ii[l] = ii[g];
                                ii[g] = 0;
                                u.iifo[l] = 0;
                                u.iifn[l] = 1;
                            }
                        }
                    }
                }
            }
        });
    }

    // Operator_Ext_LorentzMaterial::BuildExtension (operator_ext_lorentzmaterial.cpp:117-414).
    // The x planes run in parallel; each plane's position lists are joined in
    // x order, which is the reference's list order.  (The running "ADE on"
    // flag the reference tests before R_D / G_D only matters where L_D / C_D
    // is 0, and then R_D / G_D are 0 either way.)
    void BuildLorentz() {
        int order = 0;
        for (const oracle_prim& p : csx.P)
            if (p.kind == 1 && p.disp_order > order) order = p.disp_order;
        ade.assign((size_t)order, AdeO());
        struct Plane {
            std::vector<uint32_t> pos[3];
            std::vector<double> v_int[3], v_ext[3], i_int[3], i_ext[3], v_lor[3], i_lor[3];
            bool vo = false, co = false, vlo = false, clo = false;
        };
        for (int o = 0; o < order; ++o) {
            std::vector<Plane> planes(N[0]);
            parallel_x(N[0], threads, [&](uint32_t x0, uint32_t x1, int) {
                uint32_t pos[3];
                double coord[3];
                for (pos[0] = x0; pos[0] < x1; ++pos[0]) {
                    Plane& PL = planes[pos[0]];
                    for (pos[1] = 0; pos[1] < N[1]; ++pos[1]) {
                        std::vector<int> vPrims =
                            PrimitivesBoundBox((int)pos[0], (int)pos[1], -1, T_MATERIAL | T_METAL);
                        for (pos[2] = 0; pos[2] < N[2]; ++pos[2]) {
                            bool b_pos_on = false;
                            double L_D[3], R_D[3], C_L[3], C_D[3], G_D[3], L_L[3];
                            for (int n = 0; n < 3; ++n) {
                                L_D[n] = 0; R_D[n] = 0; C_L[n] = 0;
                                if (!GetYeeCoords(n, pos, coord, false)) continue;
                                if (vi[at(n, pos)] == 0) continue;
                                int w = csx.by_coord_priority(coord, vPrims);
                                if (w < 0) continue;
                                const oracle_prim& m = csx.P[w];
                                if (!(m.kind == 1 && m.disp_order > 0)) continue;
                                double ecc = EC_C[at(n, pos)];
                                double w_plasma = (o < m.disp_order ? m.eps_plasma_f[o] : 0) * 2 * kPI;
                                if ((w_plasma > 0) && (ecc > 0)) {
                                    b_pos_on = true;
                                    PL.vo = true;
                                    L_D[n] = 1 / (w_plasma * w_plasma * ecc);
                                }
                                double t_relax = o < m.disp_order ? m.eps_relax_t[o] : 0;
                                if ((t_relax > 0) && L_D[n] > 0) R_D[n] = L_D[n] / t_relax;
                                double w_Lor_Pol = (o < m.disp_order ? m.eps_pole_f[o] : 0) * 2 * kPI;
                                if ((w_Lor_Pol > 0) && (L_D[n] > 0)) {
                                    PL.vlo = true;
                                    C_L[n] = 1 / (w_Lor_Pol * w_Lor_Pol * L_D[n]);
                                }
                            }
                            for (int n = 0; n < 3; ++n) {
                                C_D[n] = 0; G_D[n] = 0; L_L[n] = 0;
                                if (!GetYeeCoords(n, pos, coord, true)) continue;
                                if (iv[at(n, pos)] == 0) continue;
                                int w = csx.by_coord_priority(coord, vPrims);
                                if (w < 0) continue;
                                const oracle_prim& m = csx.P[w];
                                if (!(m.kind == 1 && m.disp_order > 0)) continue;
                                double ecl = EC_L[at(n, pos)];
                                double w_plasma = (o < m.disp_order ? m.mue_plasma_f[o] : 0) * 2 * kPI;
                                if ((w_plasma > 0) && (ecl > 0)) {
                                    b_pos_on = true;
                                    PL.co = true;
                                    C_D[n] = 1 / (w_plasma * w_plasma * ecl);
                                }
                                double t_relax = o < m.disp_order ? m.mue_relax_t[o] : 0;
                                if ((t_relax > 0) && C_D[n] > 0) G_D[n] = C_D[n] / t_relax;
                                double w_Lor_Pol = (o < m.disp_order ? m.mue_pole_f[o] : 0) * 2 * kPI;
                                if ((w_Lor_Pol > 0) && (C_D[n] > 0)) {
                                    PL.clo = true;
                                    L_L[n] = 1 / (w_Lor_Pol * w_Lor_Pol * C_D[n]);
                                }
                            }
                            if (!b_pos_on) continue;
                            for (int n = 0; n < 3; ++n) {
                                PL.pos[n].push_back(pos[n]);
                                double VI = vi[at(n, pos)], IV = iv[at(n, pos)];
                                if (L_D[n] > 0) {
                                    PL.v_int[n].push_back((2.0 * L_D[n] - dT * R_D[n]) / (2.0 * L_D[n] + dT * R_D[n]));
                                    PL.v_ext[n].push_back(dT / (L_D[n] + dT * R_D[n] / 2.0) * VI);
                                } else if ((R_D[n] > 0) && (C_L[n] > 0)) {
                                    PL.v_int[n].push_back((2.0 * dT - R_D[n] * C_L[n]) / (C_L[n] * R_D[n]));
                                    PL.v_ext[n].push_back(2.0 / R_D[n] * VI);
                                } else {
                                    PL.v_int[n].push_back(1);
                                    PL.v_ext[n].push_back(0);
                                }
                                if (C_D[n] > 0) {
                                    PL.i_int[n].push_back((2.0 * C_D[n] - dT * G_D[n]) / (2.0 * C_D[n] + dT * G_D[n]));
                                    PL.i_ext[n].push_back(dT / (C_D[n] + dT * G_D[n] / 2.0) * IV);
                                } else {
                                    PL.i_int[n].push_back(1);
                                    PL.i_ext[n].push_back(0);
                                }
                                PL.v_lor[n].push_back(C_L[n] > 0 ? dT / C_L[n] / VI : 0);
                                PL.i_lor[n].push_back(L_L[n] > 0 ? dT / L_L[n] / IV : 0);
                            }
                        }
                    }
                }
            });
            AdeO& A = ade[(size_t)o];
            for (const Plane& PL : planes) {
                A.volt_on |= PL.vo; A.curr_on |= PL.co;
                A.volt_lor_on |= PL.vlo; A.curr_lor_on |= PL.clo;
                for (int n = 0; n < 3; ++n) A.pos[n].insert(A.pos[n].end(), PL.pos[n].begin(), PL.pos[n].end());
            }
            A.count = (uint32_t)A.pos[0].size();
            // [3][count] float arrays, NULL (empty) when that part is off
            auto fill3 = [&](std::vector<float>& dst, bool on, std::vector<double> (Plane::*m)[3]) {
                dst.clear();
                if (!on) return;
                dst.reserve(3 * (size_t)A.count);
                for (int n = 0; n < 3; ++n)
                    for (const Plane& PL : planes)
                        for (double v : (PL.*m)[n]) dst.push_back((float)v);
            };
            fill3(A.v_int, A.volt_on, &Plane::v_int);
            fill3(A.v_ext, A.volt_on, &Plane::v_ext);
            fill3(A.i_int, A.curr_on, &Plane::i_int);
            fill3(A.i_ext, A.curr_on, &Plane::i_ext);
            fill3(A.v_lor, A.volt_lor_on, &Plane::v_lor);
            fill3(A.i_lor, A.curr_lor_on, &Plane::i_lor);
        }
    }

    // Operator_Ext_LumpedRLC::BuildExtension (operator_ext_lumpedRLC.cpp:112-486)
    void BuildRLC() {
        const double fMax = f0 + fc;
        const double Z_FACT = 20.0;  // LUMPED_RLC_Z_FACT (operator_ext_lumpedRLC.h:29)
        std::vector<double> ilv, i2v, vv2, vj1, vj2, vvd, ib0v, b1v, b2v;
        for (int k : csx.by_type(T_LUMPED)) {
            const oracle_prim& P = csx.P[k];
            int dir = P.ny;
            int lumpedType = P.le_type;
            double C = P.C;
            if (C < 0) C = NAN;
            double R = P.R;
            if (R < 0) R = NAN;
            double L = P.L;
            if (L < 0) L = NAN;
            // IsLElumpedRLC: the element's own type (INVALID is neither)
            bool isParallelRLC = (P.le_type == FDTD_LE_PARALLEL) && (P.L > 0.0);
            bool isSeriesRLC = P.le_type == FDTD_LE_SERIES;
            if (!(isParallelRLC || isSeriesRLC)) continue;
            if (lumpedType == FDTD_LE_INVALID) lumpedType = FDTD_LE_PARALLEL;
            if (dir < 0 || dir > 2) continue;
            int dir_p1 = (dir + 1) % 3, dir_p2 = (dir + 2) % 3;
            uint32_t uiStart[3], uiStop[3];
            int dim = SnapBox2Mesh(P.start, P.stop, uiStart, uiStop, false, 0);
            if (dim <= 0) continue;
            if (uiStart[dir] == uiStop[dir]) continue;
            uint32_t Ncells_0 = uiStop[dir] - uiStart[dir];
            uint32_t Ncells_1 = uiStop[dir_p1] - uiStart[dir_p1] + 1;
            uint32_t Ncells_2 = uiStop[dir_p2] - uiStart[dir_p2] + 1;
            uint32_t Npar = Ncells_1 * Ncells_2;
            double dL = L * Npar / Ncells_0, dR = R * Npar / Ncells_0, dG = (1 / R) * Ncells_0 / Npar,
                   dC = C * Ncells_0 / Npar;
            double ib0 = 2.0 * dT * dC / (4.0 * dL * dC + 2.0 * dT * dR * dC + dT * dT),
                   b1 = (dT * dT - 4.0 * dL * dC) / (dT * dC),
                   b2 = (4.0 * dL * dC - 2.0 * dT * dR * dC + dT * dT) / (2.0 * dT * dC);
            if (lumpedType == FDTD_LE_PARALLEL)
                if (R == 0.0) dG = 0.0;
            uint32_t pos[3];
            double Zmin, Zcd_min;
            for (pos[dir] = uiStart[dir]; pos[dir] < uiStop[dir]; ++pos[dir])
                for (pos[dir_p1] = uiStart[dir_p1]; pos[dir_p1] <= uiStop[dir_p1]; ++pos[dir_p1])
                    for (pos[dir_p2] = uiStart[dir_p2]; pos[dir_p2] <= uiStop[dir_p2]; ++pos[dir_p2]) {
                        size_t iPos = at(dir, pos);
                        if (lumpedType == FDTD_LE_PARALLEL) {
                            if (dC > 0)
                                EC_C[iPos] = (float)dC;
                            else
                                dC = EC_C[iPos];
                            i2v.push_back((dT / dC) / (1.0 + dT * dG / (2.0 * dC)));
                            if (R >= 0) EC_G[iPos] = (float)dG;
                            if (L > 0)
                                ilv.push_back(dT / dL);
                            else
                                ilv.push_back(0.0);
                            if (dC == 0) {
                                double Cd = EC_C[iPos];
                                Zmin = std::max(dR, 2 * kPI * fMax * dL);
                                Zcd_min = 1.0 / (2.0 * kPI * fMax * Cd);
                                if (Zcd_min < Z_FACT * Zmin) {
                                    Cd = 1.0 / (2 * kPI * fMax * Zmin * Z_FACT);
                                    EC_C[iPos] = (float)Cd;
                                }
                            }
                            vv2.push_back(0.0); vj1.push_back(0.0); vj2.push_back(0.0); vvd.push_back(1.0);
                            ib0v.push_back(0.0); b1v.push_back(0.0); b2v.push_back(0.0);
                            Calc_ECOperatorPos(dir, pos);
                            r_dir.push_back(dir);
                        } else {  // SERIES
                            EC_G[iPos] = 0.0f;
                            float Cd = EC_C[iPos];
                            Zmin = std::sqrt(std::pow(dR, 2) + std::pow(2 * kPI * fMax * dL - 1.0 / (dC * 2 * kPI * fMax), 2));
                            Zcd_min = 1.0 / (2.0 * kPI * fMax * Cd);
                            if (Zcd_min < Z_FACT * Zmin) {
                                Cd = (float)(1.0 / (2 * kPI * fMax * Zmin * Z_FACT));
                                EC_C[iPos] = Cd;
                            }
                            ilv.push_back(0.0);
                            i2v.push_back(0.0);
                            vv2.push_back(0.5 * dT * ib0 / Cd);
                            vj1.push_back(0.5 * dT * (b1 * ib0 - 1.0) / Cd);
                            vj2.push_back(0.5 * dT * b2 * ib0 / Cd);
                            vvd.push_back(1.0 / (1.0 + 0.5 * dT * ib0 / Cd));
                            ib0v.push_back(ib0);
                            b1v.push_back(b1);
                            b2v.push_back(b2);
                            Calc_ECOperatorPos(dir, pos);
                            r_dir.push_back(dir);
                        }
                        for (int a = 0; a < 3; ++a) r_pos[a].push_back(pos[a]);
                    }
            if (P.caps)
                for (pos[dir_p1] = uiStart[dir_p1]; pos[dir_p1] <= uiStop[dir_p1]; ++pos[dir_p1])
                    for (pos[dir_p2] = uiStart[dir_p2]; pos[dir_p2] <= uiStop[dir_p2]; ++pos[dir_p2]) {
                        pos[dir] = uiStart[dir];
                        if (pos[dir_p1] < uiStop[dir_p1]) { SetVV(dir_p1, pos, 0); SetVI(dir_p1, pos, 0); }
                        if (pos[dir_p2] < uiStop[dir_p2]) { SetVV(dir_p2, pos, 0); SetVI(dir_p2, pos, 0); }
                        pos[dir] = uiStop[dir];
                        if (pos[dir_p1] < uiStop[dir_p1]) { SetVV(dir_p1, pos, 0); SetVI(dir_p1, pos, 0); }
                        if (pos[dir_p2] < uiStop[dir_p2]) { SetVV(dir_p2, pos, 0); SetVI(dir_p2, pos, 0); }
                    }
        }
        auto cvt = [](const std::vector<double>& s, std::vector<float>& d) {
            d.resize(s.size());
            for (size_t i = 0; i < s.size(); ++i) d[i] = (float)s[i];
        };
        cvt(ilv, r_ilv); cvt(i2v, r_i2v); cvt(vv2, r_vv2); cvt(vj1, r_vj1); cvt(vj2, r_vj2);
        cvt(vvd, r_vvd); cvt(ib0v, r_ib0); cvt(b1v, r_b1); cvt(b2v, r_b2);
    }

    // CalcNyquistNum (tools/useful.cpp:30-36)
    uint32_t CalcNyquistNum(double fmax) const {
        if (fmax == 0) return UINT_MAX;
        if (dT == 0) return 1;
        double T0 = 1 / fmax;
        return (uint32_t)std::floor(T0 / 2 / dT);
    }
    // Excitation::CalcGaussianPulsExcitation (excitation.cpp:151-177)
    void CalcGaussianPulsExcitation() {
        length = (uint32_t)std::ceil(2.0 * 9.0 / (2.0 * kPI * fc) / dT);
        if (length > nr_ts) length = nr_ts;
        sig_v.resize(length);
        sig_c.resize(length);
        for (uint32_t n = 0; n < length; ++n) {
            double t = n * dT;
            sig_v[n] = (float)(std::cos(2.0 * kPI * f0 * (t - 9.0 / (2.0 * kPI * fc))) *
                               std::exp(-1 * std::pow(2.0 * kPI * fc * t / 3.0 - 3, 2)));
            t += 0.5 * dT;
            sig_c[n] = (float)(std::cos(2.0 * kPI * f0 * (t - 9.0 / (2.0 * kPI * fc))) *
                               std::exp(-1 * std::pow(2.0 * kPI * fc * t / 3.0 - 3, 2)));
        }
        nyquist = CalcNyquistNum(f0 + fc);
    }
    // Excitation::CalcSinusExcitation (excitation.cpp:273-295)
    void CalcSinusExcitation() {
        length = (uint32_t)std::round(2.0 / f0 / dT);
        sig_v.resize(length);
        sig_c.resize(length);
        if (length) sig_v[0] = 0.0f, sig_c[0] = 0.0f;
        for (uint32_t n = 1; n < length; ++n) {
            double t = n * dT;
            sig_v[n] = (float)std::sin(2.0 * kPI * f0 * t);
            t += 0.5 * dT;
            sig_c[n] = (float)std::sin(2.0 * kPI * f0 * t);
        }
        nyquist = CalcNyquistNum(f0);
    }
    // Excitation::CalcDiracPulsExcitation / CalcStepExcitation (excitation.cpp:179-218)
    void CalcUnitExcitation(bool step) {
        length = 2;
        sig_v = {step ? 1.0f : 0.0f, 1.0f};
        sig_c = {step ? 1.0f : 0.0f, 1.0f};
        nyquist = 1;
    }
    // Excitation::CalcCustomExcitation (excitation.cpp:233-271)
    bool CalcCustomExcitation() {
        OracleFunction F;
        if (!F.parse(function)) return false;
        length = nr_ts;
        sig_v.resize(length);
        sig_c.resize(length);
        double vars[1];
        for (uint32_t n = 0; n < length; ++n) {
            vars[0] = n * dT;
            sig_v[n] = (float)F.eval(vars[0]);
            vars[0] += 0.5 * dT;
            sig_c[n] = (float)F.eval(vars[0]);
        }
        nyquist = CalcNyquistNum(f0);
        return true;
    }
    // Excitation::buildExcitationSignal (excitation.cpp:96-134)
    bool BuildSignal() {
        switch (excite_type) {
            case 0: CalcGaussianPulsExcitation(); break;
            case 1: CalcSinusExcitation(); break;
            case 10: if (!CalcCustomExcitation()) return false; break;
            default: CalcUnitExcitation(excite_type == 3); break;
        }
        // Engine_Ext_Excitation's period (engine_ext_excitation.cpp:44-46)
        period_ts = signal_period > 0 ? (uint32_t)int(signal_period / dT) : 0;
        // Excitation::GetMaxExcitationTimestep (excitation.cpp:136-149)
        float maxAmp = 0;
        max_exc_ts = 0;
        for (uint32_t n = 0; n < length; ++n)
            if (std::fabs(sig_v[n]) > maxAmp) {
                maxAmp = std::fabs(sig_v[n]);
                max_exc_ts = n;
            }
        return true;
    }

    // openEMS::SetupProcessing probe loop (openems.cpp:470-540)
    void SetupProbes() {
        uint32_t interval = oversampling ? nyquist / oversampling : nyquist;
        probe_interval = std::max(1u, interval);
        for (int k : csx.by_type(T_PROBE)) {
            const oracle_prim& P = csx.P[k];
            fdtd_probe_desc d;
            std::memset(&d, 0, sizeof(d));
            d.type = P.probe_type;
            d.weight = P.weight;
            d.norm_dir = P.norm_dir;
            d.enabled = 1;
            double start[3], stop[3];
            for (int n = 0; n < 3; ++n) {
                start[n] = std::fmin(P.start[n], P.stop[n]);
                stop[n] = std::fmax(P.start[n], P.stop[n]);
            }
            bool sin[3] = {false, false, false}, ein[3] = {false, false, false};
            if (P.probe_type == 0) {
                int dimension = 0;
                for (int n = 0; n < 3; ++n)
                    if (P.start[n] != P.stop[n]) ++dimension;
                if (dimension != 1) continue;  // "Probe primitive type or dimension not suitable"
                // ProcessVoltage::DefineStartStopCoord: the box's own start / stop, main mesh
                SnapToMesh(P.start, d.start, false, sin);
                SnapToMesh(P.stop, d.stop, false, ein);
            } else if (P.probe_type == 1) {
                // Processing::DefineStartStopCoord (snap method 1, dual mesh), then ProcessCurrent
                int dim = SnapBox2Mesh(start, stop, d.start, d.stop, true, 1, sin, ein);
                if (dim < 0) d.enabled = 0;
                int normDir = P.norm_dir;
                if ((normDir < 0) || (normDir > 2)) {
                    if (dim != 2) {
                        d.enabled = 0;
                    } else {
                        for (int n = 0; n < 3; ++n)
                            if (d.stop[n] == d.start[n]) normDir = n;
                    }
                } else {
                    dim = 0;
                    for (int n = 0; n < 3; ++n) {
                        if (n == normDir) continue;
                        if (start[n] == stop[n]) {
                            if ((GetDiscLine(n, d.start[n], true) > start[n]) && (d.start[n] > 0)) --d.start[n];
                            if ((GetDiscLine(n, d.start[n], true) < start[n]) && (d.stop[n] < N[n] - 1)) ++d.stop[n];
                        }
                        if (d.stop[n] > d.start[n]) ++dim;
                    }
                }
                if (d.enabled && normDir >= 0 && normDir <= 2 && d.start[normDir] != d.stop[normDir]) d.enabled = 0;
                if (d.enabled && (normDir < 0 || normDir > 2)) d.enabled = 0;
                d.norm_dir = normDir;
            } else if (P.probe_type == 2 || P.probe_type == 3) {
                int dim = SnapBox2Mesh(start, stop, d.start, d.stop, P.probe_type == 3, 0, sin, ein);
                if (dim < 0) d.enabled = 0;
            } else {
                continue;
            }
            for (int n = 0; n < 3; ++n) {
                d.start_inside[n] = sin[n];
                d.stop_inside[n] = ein[n];
            }
            probes.push_back(d);
        }
    }

    // Operator::CalcECOperator (operator.cpp:973-1084) + the extension builds
    // in the order openEMS adds them + Excitation::buildExcitationSignal
    int build() {
        Calc_EC();
        dT = CalcTimestep_Var3();
        if (!(dT > 0) || dT >= 1e200) return -1;
        // m_TimeStepFactor 1; a periodic signal fits a whole number of
        // timesteps into its period (operator.cpp:999-1007)
        if (signal_period > 0) {
            unsigned int TS = (unsigned int)std::ceil(signal_period / dT);
            double new_dT = signal_period / TS;
            dT = new_dT;
        }
        vv.assign(3 * NN, 0.f);
        vi.assign(3 * NN, 0.f);
        ii.assign(3 * NN, 0.f);
        iv.assign(3 * NN, 0.f);
        parallel_x(N[0], threads, [&](uint32_t x0, uint32_t x1, int) {
            uint32_t pos[3];
            for (int n = 0; n < 3; ++n)
                for (pos[0] = x0; pos[0] < x1; ++pos[0])
                    for (pos[1] = 0; pos[1] < N[1]; ++pos[1])
                        for (pos[2] = 0; pos[2] < N[2]; ++pos[2]) Calc_ECOperatorPos(n, pos);
        });
        bool PEC[6], PMC[6];
        for (int n = 0; n < 6; ++n) PEC[n] = BC[n] != -1;
        ApplyElectricBC(PEC);
        CalcPEC();
        Calc_LumpedElements();
        for (int n = 0; n < 6; ++n) PMC[n] = BC[n] == 1;
        ApplyMagneticBC(PMC);

        // extensions: excitation, Mur faces, UPML slabs, Lorentz, lumped RLC
        BuildExcitation();
        for (int k = 0; k < 6; ++k) {
            if (BC[k] != 2) continue;
            MurO M;
            M.ny = k / 2;
            M.top = (k % 2) != 0;
            M.nyP = (M.ny + 1) % 3;
            M.nyPP = (M.ny + 2) % 3;
            M.line = M.top ? N[M.ny] - 1 : 0;
            M.shift = M.top ? N[M.ny] - 2 : 1;
            M.nl[0] = N[M.nyP];
            M.nl[1] = N[M.nyPP];
            M.vph = mur_vph[k];
            BuildMur(M);
            mur.push_back(std::move(M));
        }
        if (!CreateUPML()) return -3;
        for (UpmlSlabO& u : upml) BuildUPML(u);
        bool have_lorentz = false;
        for (const oracle_prim& p : csx.P)
            if (p.kind == 1 && p.disp_order > 0) have_lorentz = true;
        if (have_lorentz) BuildLorentz();
        if (!csx.by_type(T_LUMPED).empty()) BuildRLC();

        if (!BuildSignal()) return -1;
        // Engine_Ext_Mur_ABC start timestep (engine_ext_mur_abc.cpp:43-58)
        for (MurO& M : mur) {
            int maxDelay = -1;
            for (size_t n = 0; n < v_amp.size(); ++n)
                if (((v_dir[n] == M.nyP) || (v_dir[n] == M.nyPP)) && (v_idx[M.ny][n] == M.line))
                    if ((int)v_delay[n] > maxDelay) maxDelay = (int)v_delay[n];
            M.start_ts = maxDelay >= 0 ? (uint32_t)maxDelay + length + 10 : 0;
        }
        SetupProbes();
        return 0;
    }
};

extern "C" {

int oracle_operator_build(const oracle_scene* S, int threads, oracle_operator_s** out) {
    if (!S || !out) return -1;
    std::unique_ptr<oracle_operator_s> op(new oracle_operator_s());
    for (int n = 0; n < 3; ++n) {
        if (S->num_lines[n] < 2 || !S->lines[n]) return -1;
        op->N[n] = S->num_lines[n];
        op->lines[n].assign(S->lines[n], S->lines[n] + S->num_lines[n]);
    }
    op->NN = (size_t)op->N[0] * op->N[1] * op->N[2];
    op->unit = S->unit;
    op->bg[0] = S->bg_eps;
    op->bg[1] = S->bg_kappa;
    op->bg[2] = S->bg_mue;
    op->bg[3] = S->bg_sigma;
    for (int k = 0; k < 6; ++k) {
        op->BC[k] = S->bc[k];
        // a face that is not PML keeps openEMS's default size 8
        // (openems.cpp:101), which Create_UPML / CalcGradingKappa still read
        op->pml[k] = S->bc[k] == 3 ? S->pml_size[k] : 8;
        op->mur_vph[k] = S->mur_vph[k];
    }
    // openEMS::Parse_XML_FDTDSetup / Excitation::Setup* (openems.cpp:900-927,
    // excitation.cpp:56-85): the Dirac and step leave m_f0 / m_fc unset in
    // the reference; 0 here
    op->excite_type = S->excite_type;
    op->function = S->function ? S->function : "";
    op->f0 = (S->excite_type <= 1 || S->excite_type == 10) ? S->f0 : 0.0;
    op->fc = S->excite_type == 0 ? S->fc : 0.0;
    op->signal_period = S->excite_type == 1 ? 1 / S->f0 : 0.0;
    op->nr_ts = S->nr_ts;
    op->oversampling = S->oversampling ? S->oversampling : 4;
    op->threads = threads > 0 ? threads : (int)std::max(1u, std::thread::hardware_concurrency());
    op->csx.P.assign(S->prims, S->prims + S->num_prims);
    op->csx.init();
    try {
        const int rc = op->build();
        if (rc != 0) return rc == -3 ? -3 : -2;
    } catch (const std::bad_alloc&) {
        return -4;
    }
    *out = op.release();
    return 0;
}

void oracle_operator_destroy(oracle_operator_s* op) { delete op; }

int oracle_operator_info(const oracle_operator_s* op, oracle_op_info* info) {
    if (!op || !info) return -1;
    for (int n = 0; n < 3; ++n) info->num_lines[n] = op->N[n];
    info->dT = op->dT;
    info->nyquist = op->nyquist;
    info->probe_interval = op->probe_interval;
    info->signal_length = op->length;
    info->max_excite_ts = op->max_exc_ts;
    info->num_probes = (uint32_t)op->probes.size();
    return 0;
}

int oracle_operator_probe(const oracle_operator_s* op, uint32_t i, fdtd_probe_desc* out) {
    if (!op || !out || i >= op->probes.size()) return -1;
    *out = op->probes[i];
    return 0;
}

// Fills the engine description (the layout of include/wipems_fdtd.h) with
// pointers into the oracle operator's arrays.
int oracle_operator_describe(oracle_operator_s* op, fdtd_op_desc* d) {
    if (!op || !d) return -1;
    std::memset(d, 0, sizeof(*d));
    for (int n = 0; n < 3; ++n) d->num_lines[n] = op->N[n];
    d->dT = op->dT;
    d->vv = op->vv.data();
    d->vi = op->vi.data();
    d->ii = op->ii.data();
    d->iv = op->iv.data();
    op->upml_desc.resize(op->upml.size());
    for (size_t k = 0; k < op->upml.size(); ++k) {
        const UpmlSlabO& s = op->upml[k];
        fdtd_upml_desc& u = op->upml_desc[k];
        for (int n = 0; n < 3; ++n) {
            u.start[n] = s.start[n];
            u.num_lines[n] = s.nl[n];
        }
        u.vv = s.vv.data(); u.vvfo = s.vvfo.data(); u.vvfn = s.vvfn.data();
        u.ii = s.ii.data(); u.iifo = s.iifo.data(); u.iifn = s.iifn.data();
    }
    d->num_upml = (uint32_t)op->upml.size();
    d->upml = op->upml_desc.empty() ? nullptr : op->upml_desc.data();
    op->ade_desc.resize(op->ade.size());
    for (size_t k = 0; k < op->ade.size(); ++k) {
        const AdeO& s = op->ade[k];
        fdtd_ade_desc& a = op->ade_desc[k];
        a.count = s.count;
        for (int n = 0; n < 3; ++n) a.pos[n] = s.pos[n].data();
        a.volt_on = s.volt_on; a.curr_on = s.curr_on;
        a.volt_lor_on = s.volt_lor_on; a.curr_lor_on = s.curr_lor_on;
        a.v_int = s.v_int.empty() ? nullptr : s.v_int.data();
        a.v_ext = s.v_ext.empty() ? nullptr : s.v_ext.data();
        a.v_lor = s.v_lor.empty() ? nullptr : s.v_lor.data();
        a.i_int = s.i_int.empty() ? nullptr : s.i_int.data();
        a.i_ext = s.i_ext.empty() ? nullptr : s.i_ext.data();
        a.i_lor = s.i_lor.empty() ? nullptr : s.i_lor.data();
    }
    d->num_ade_orders = (uint32_t)op->ade.size();
    d->ade = op->ade_desc.empty() ? nullptr : op->ade_desc.data();
    d->volt_count = (uint32_t)op->v_amp.size();
    d->curr_count = (uint32_t)op->c_amp.size();
    for (int n = 0; n < 3; ++n) {
        d->volt_index[n] = op->v_idx[n].data();
        d->curr_index[n] = op->c_idx[n].data();
    }
    d->volt_dir = op->v_dir.data();
    d->volt_amp = op->v_amp.data();
    d->volt_delay = op->v_delay.data();
    d->curr_dir = op->c_dir.data();
    d->curr_amp = op->c_amp.data();
    d->curr_delay = op->c_delay.data();
    op->mur_desc.resize(op->mur.size());
    for (size_t k = 0; k < op->mur.size(); ++k) {
        const MurO& M = op->mur[k];
        fdtd_mur_desc& m = op->mur_desc[k];
        m.ny = M.ny;
        m.top = M.top ? 1 : 0;
        m.line = M.line;
        m.shift = M.shift;
        m.n_p = M.nl[0];
        m.n_pp = M.nl[1];
        m.coef_p = M.cp.data();
        m.coef_pp = M.cpp.data();
        m.start_ts = M.start_ts;
    }
    d->num_mur = (uint32_t)op->mur.size();
    d->mur = op->mur_desc.empty() ? nullptr : op->mur_desc.data();
    fdtd_rlc_desc& q = op->rlc_desc;
    q.count = (uint32_t)op->r_dir.size();
    for (int n = 0; n < 3; ++n) q.pos[n] = op->r_pos[n].data();
    q.dir = op->r_dir.data();
    q.ilv = op->r_ilv.data(); q.i2v = op->r_i2v.data();
    q.vv2 = op->r_vv2.data(); q.vj1 = op->r_vj1.data(); q.vj2 = op->r_vj2.data(); q.vvd = op->r_vvd.data();
    q.ib0 = op->r_ib0.data(); q.b1 = op->r_b1.data(); q.b2 = op->r_b2.data();
    d->rlc = q.count ? &op->rlc_desc : nullptr;
    d->signal_length = op->length;
    d->signal_volt = op->sig_v.data();
    d->signal_curr = op->sig_c.data();
    d->signal_period_ts = op->period_ts;
    for (int n = 0; n < 3; ++n) d->lines[n] = op->lines[n].data();
    d->unit = op->unit;
    return 0;
}

}  // extern "C"
