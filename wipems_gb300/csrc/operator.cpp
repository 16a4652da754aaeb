// Host-side FDTD operator build: the equivalent-circuit coefficients of every
// Yee edge, computed from a scene of priority-ordered boxes.
//
// This restates openEMS's setup path (all citations relative to the
// reference project):
//   Operator::CalcECOperator          FDTD/operator.cpp:973-1084
//   Operator::Calc_ECPos              FDTD/operator.cpp:1176-1224
//   Operator::AverageMatQuarterCell   FDTD/operator.cpp:1406-1518
//   Operator::Calc_ECOperatorPos      FDTD/operator.cpp:943-971
//   Operator::CalcTimestep_Var3       FDTD/operator.cpp:1897-1971
//   Operator::ApplyElectricBC/MagneticBC FDTD/operator.cpp:1086-1174
//   Operator::CalcPEC_Range           FDTD/operator.cpp:1986-2020
//   Operator::Calc_LumpedElements     FDTD/operator.cpp:1535-1712
//   Operator_Ext_Excitation::BuildExtension operator_ext_excitation.cpp:101-285
//   Operator_Ext_UPML::Create_UPML / CalcGradingKappa / BuildExtension
//                                     operator_ext_upml.cpp:77-466
//   Operator_Ext_LorentzMaterial::BuildExtension
//                                     operator_ext_lorentzmaterial.cpp:117-438
//   Excitation::CalcGaussianPulsExcitation FDTD/excitation.cpp:151-177
//   Processing / ProcessCurrent / ProcessVoltage snapping
//                                     Common/processing.cpp:180-189,
//                                     processcurrent.cpp:39-91,
//                                     processvoltage.cpp:34-38
// The arithmetic is kept in the reference's order and precision (double
// math, FP32 storage of the EC arrays and of the coefficients) so that the
// resulting FP32 tables are the ones the reference engine would step with.
//
// CSXCAD (absent from the reference tree) is replaced by a box model:
// GetPropertyByCoordPriority picks the highest-priority box containing the
// coordinate (surface included; first-added wins on equal priority), and all
// *Weighted material getters return the box's constant value.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <functional>
#include <limits>
#include <memory>
#include <thread>

#include "fdtd_host.h"
#include "signal_expr.h"

namespace wipems {

namespace {

thread_local std::string g_last_error;

// ---------------------------------------------------------------- geometry
// Mesh helpers of Operator (operator.cpp:136-242, 1226-1236).
struct Geo {
    const std::vector<double>* L;  // lines[3], drawing units
    uint32_t N[3];
    double unit;

    double line(int n, uint32_t pos, bool dual) const {  // GetDiscLine
        if (pos >= N[n]) return 0.0;
        const std::vector<double>& l = L[n];
        if (!dual) return l[pos];
        if (pos < N[n] - 1) return 0.5 * (l[pos] + l[pos + 1]);
        return l[pos] + 0.5 * (l[pos] - l[pos - 1]);
    }
    // GetDiscDelta per axis and mesh, evaluated once (cache()) and then read
    std::vector<double> dd[3][2];
    void cache() {
        for (int n = 0; n < 3; ++n)
            for (int d = 0; d < 2; ++d) {
                dd[n][d].clear();
                std::vector<double> v(N[n]);
                for (uint32_t i = 0; i < N[n]; ++i) v[i] = disc_delta_eval(n, i, d != 0);
                dd[n][d] = std::move(v);
            }
    }
    double disc_delta(int n, uint32_t pos, bool dual) const {
        if (pos >= N[n]) return 0.0;
        const std::vector<double>& c = dd[n][dual ? 1 : 0];
        if (!c.empty()) return c[pos];
        return disc_delta_eval(n, pos, dual);
    }
    double disc_delta_eval(int n, uint32_t pos, bool dual) const {  // GetDiscDelta
        if (pos >= N[n]) return 0.0;
        double delta = 0;
        if (!dual) {
            if (pos < N[n] - 1)
                delta = line(n, pos + 1, false) - line(n, pos, false);
            else
                delta = line(n, pos, false) - line(n, pos - 1, false);
            return delta;
        }
        if (pos > 0)
            delta = line(n, pos, true) - line(n, pos - 1, true);
        else
            delta = line(n, 1, false) - line(n, 0, false);
        return delta;
    }
    double edge_length(int n, const uint32_t* pos, bool dual) const {  // GetEdgeLength
        return disc_delta(n, pos[n], dual) * unit;
    }
    double node_width(int n, const uint32_t* pos, bool dual) const {  // GetNodeWidth
        return edge_length(n, pos, !dual);
    }
    double node_width_i(int n, const int* pos, bool dual) const {
        if (pos[0] < 0 || pos[1] < 0 || pos[2] < 0) return 0.0;
        uint32_t u[3] = {(uint32_t)pos[0], (uint32_t)pos[1], (uint32_t)pos[2]};
        return node_width(n, u, dual);
    }
    double node_area(int ny, const uint32_t* pos, bool dual) const {  // GetNodeArea
        int nyP = (ny + 1) % 3, nyPP = (ny + 2) % 3;
        return node_width(nyP, pos, dual) * node_width(nyPP, pos, dual);
    }
    double node_area_i(int ny, const int* pos, bool dual) const {
        if (pos[0] < 0 || pos[1] < 0 || pos[2] < 0) return 0.0;
        uint32_t u[3] = {(uint32_t)pos[0], (uint32_t)pos[1], (uint32_t)pos[2]};
        return node_area(ny, u, dual);
    }
    double edge_area(int ny, const uint32_t* pos, bool dual) const {  // GetEdgeArea
        return node_area(ny, pos, dual);
    }
    double raw_delta(int ny, int pos) const {  // GetRawDiscDelta
        const std::vector<double>& l = L[ny];
        if (pos < 0) return l[0] - l[1];
        if (pos >= (int)N[ny] - 1) return l[N[ny] - 2] - l[N[ny] - 1];
        return l[pos + 1] - l[pos];
    }
    // GetYeeCoords: returns false when outside the FDTD domain.
    bool yee_coords(int ny, const uint32_t* pos, double* c, bool dual) const {
        for (int n = 0; n < 3; ++n) c[n] = line(n, pos[n], dual);
        c[ny] = line(ny, pos[ny], !dual);
        if (!dual) return !(pos[ny] >= N[ny] - 1);
        int nP = (ny + 1) % 3, nPP = (ny + 2) % 3;
        return !((pos[nP] >= N[nP] - 1) || (pos[nPP] >= N[nPP] - 1));
    }
    // SnapToMeshLine (operator.cpp:244-272)
    uint32_t snap_line(int ny, double coord, bool& inside, bool dual) const {
        inside = false;
        if (coord < line(ny, 0, false)) return 0;
        uint32_t nl = N[ny];
        if (coord > line(ny, nl - 1, false)) return nl - 1;
        inside = true;
        if (!dual) {
            for (uint32_t n = 0; n < nl; ++n)
                if (coord <= line(ny, n, true)) return n;
        } else {
            for (uint32_t n = 1; n < nl; ++n)
                if (coord <= line(ny, n, false)) return n - 1;
        }
        return 0;
    }
    bool snap_mesh(const double* dc, uint32_t* ui, bool dual, bool* inside) const {
        bool ok = true;
        for (int n = 0; n < 3; ++n) {
            bool in = false;
            ui[n] = snap_line(n, dc[n], in, dual);
            ok &= in;
            if (inside) inside[n] = in;
        }
        return ok;
    }
    // SnapBox2Mesh (operator.cpp:288-348)
    int snap_box(const double* start, const double* stop, uint32_t* uiStart, uint32_t* uiStop,
                 bool dual, int method, bool* bStartIn, bool* bStopIn) const {
        double ls[3], le[3];
        for (int n = 0; n < 3; ++n) {
            ls[n] = std::fmin(start[n], stop[n]);
            le[n] = std::fmax(start[n], stop[n]);
            double mn = line(n, 0, false), mx = line(n, N[n] - 1, false);
            if (((ls[n] < mn) && (le[n] < mn)) || ((ls[n] > mx) && (le[n] > mx))) return -2;
        }
        snap_mesh(ls, uiStart, dual, bStartIn);
        snap_mesh(le, uiStop, dual, bStopIn);
        int iDim = 0;
        if (method == 0) {
            for (int n = 0; n < 3; ++n)
                if (uiStop[n] > uiStart[n]) ++iDim;
            return iDim;
        }
        if (method == 1) {
            for (int n = 0; n < 3; ++n) {
                if (uiStop[n] > uiStart[n]) {
                    if ((line(n, uiStart[n], dual) > ls[n]) && (uiStart[n] > 0)) --uiStart[n];
                    if ((line(n, uiStop[n], dual) < le[n]) && (uiStop[n] < N[n] - 1)) ++uiStop[n];
                }
                if (uiStop[n] > uiStart[n]) ++iDim;
            }
            return iDim;
        }
        if (method == 2) {
            for (int n = 0; n < 3; ++n) {
                if (uiStop[n] > uiStart[n]) {
                    if ((line(n, uiStart[n], dual) < ls[n]) && (uiStart[n] < N[n] - 1)) ++uiStart[n];
                    if ((line(n, uiStop[n], dual) > le[n]) && (uiStop[n] > 0)) --uiStop[n];
                }
                if (uiStop[n] > uiStart[n]) ++iDim;
            }
            return iDim;
        }
        return -1;
    }
};

// ------------------------------------------------------ box priority lookup
// Sample coordinate kinds used by the reference's lookups, per axis and line:
//   LINE  l[i]                         (GetYeeCoords main mesh, non-edge axes)
//   DUAL  GetDiscLine(i, dual)         (edge axis of GetYeeCoords, dual mesh)
//   HALF  l[i] + raw(i)*0.5            (quarter-cell averaging)
//   QP    l[i] + raw(i)*0.25
//   QM    l[i] - raw(i-1)*0.25
//   MURLO / MURHI  l[i] +- |edge length| / 2  (Mur face material probe,
//                  operator_ext_mur_abc.cpp:132-136; used at the first /
//                  last line)
enum SampleKind { SK_LINE = 0, SK_DUAL = 1, SK_HALF = 2, SK_QP = 3, SK_QM = 4, SK_MURLO = 5, SK_MURHI = 6, SK_COUNT = 7 };

struct BoxIndex {
    std::vector<int> prim;  // bit -> prim index (priority descending, stable)
    int W = 0;              // 64-bit words per mask
    std::vector<uint64_t> masks[3][SK_COUNT];  // [axis][kind][line*W + w]

    void build(const std::vector<Prim>& prims, const std::function<bool(const Prim&)>& filter,
               const Geo& g) {
        prim.clear();
        for (size_t i = 0; i < prims.size(); ++i)
            if (filter(prims[i])) prim.push_back((int)i);
        std::stable_sort(prim.begin(), prim.end(), [&](int a, int b) {
            return prims[a].priority > prims[b].priority;
        });
        W = (int)((prim.size() + 63) / 64);
        if (W == 0) W = 1;
        for (int a = 0; a < 3; ++a) {
            uint32_t n = g.N[a];
            for (int k = 0; k < SK_COUNT; ++k) {
                masks[a][k].assign((size_t)n * W, 0);
                for (uint32_t i = 0; i < n; ++i) {
                    double c = sample(g, a, k, i);
                    for (size_t b = 0; b < prim.size(); ++b) {
                        const Prim& p = prims[prim[b]];
                        if (c >= p.bmin[a] && c <= p.bmax[a])
                            masks[a][k][(size_t)i * W + b / 64] |= (uint64_t)1 << (b % 64);
                    }
                }
            }
        }
    }
    static double sample(const Geo& g, int a, int kind, uint32_t i) {
        const std::vector<double>& l = g.L[a];
        switch (kind) {
            case SK_LINE: return l[i];
            case SK_DUAL: return g.line(a, i, true);
            case SK_HALF: return l[i] + g.raw_delta(a, (int)i) * 0.5;
            case SK_QP: return l[i] + g.raw_delta(a, (int)i) * 0.25;
            case SK_MURLO:
            case SK_MURHI: {
                const double d = std::fabs(g.disc_delta(a, i, false) * g.unit);
                return kind == SK_MURLO ? g.line(a, i, false) + d / 2 / g.unit : g.line(a, i, false) - d / 2 / g.unit;
            }
            default: return l[i] - g.raw_delta(a, (int)i - 1) * 0.25;
        }
    }
    // index range [lo, hi] of axis a in which some box matches some sample
    // kind (lookup returns -1 outside it); false when there is none
    bool span(int a, uint32_t& lo, uint32_t& hi) const {
        bool any = false;
        lo = 0;
        hi = 0;
        if (prim.empty()) return false;
        for (int k = 0; k < SK_COUNT; ++k) {
            const std::vector<uint64_t>& m = masks[a][k];
            const size_t n = m.size() / (size_t)W;
            for (size_t i = 0; i < n; ++i) {
                bool hit = false;
                for (int w = 0; w < W; ++w) hit |= m[i * W + w] != 0;
                if (!hit) continue;
                if (!any || i < lo) lo = (uint32_t)i;
                if (!any || i > hi) hi = (uint32_t)i;
                any = true;
            }
        }
        return any;
    }
    // winner for (kind,index) per axis; -1 = none
    int lookup(const int kind[3], const uint32_t idx[3]) const {
        if (prim.empty()) return -1;
        const uint64_t* m0 = &masks[0][kind[0]][(size_t)idx[0] * W];
        const uint64_t* m1 = &masks[1][kind[1]][(size_t)idx[1] * W];
        const uint64_t* m2 = &masks[2][kind[2]][(size_t)idx[2] * W];
        for (int w = 0; w < W; ++w) {
            uint64_t m = m0[w] & m1[w] & m2[w];
            if (m) return prim[w * 64 + __builtin_ctzll(m)];
        }
        return -1;
    }
};

bool is_material(const Prim& p) { return p.kind == PK_MATERIAL; }
bool is_mat_or_metal(const Prim& p) { return p.kind == PK_MATERIAL || p.kind == PK_METAL; }
bool is_excitation(const Prim& p) { return p.kind == PK_EXCITATION; }

// f(i, thread) for i in [0, n); the threads take `grain` consecutive
// indices at a time (short items: fewer shared-counter round trips, and no
// two threads writing neighbouring items' cache lines)
template <class F>
void parallel_for(uint32_t n, int threads, F&& f, uint32_t grain = 1) {
    if (threads <= 1 || n < 2) {
        for (uint32_t i = 0; i < n; ++i) f(i, 0);
        return;
    }
    if (grain < 1) grain = 1;
    std::atomic<uint32_t> next{0};
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t)
        pool.emplace_back([&, t] {
            for (;;) {
                const uint32_t i0 = next.fetch_add(grain);
                if (i0 >= n) break;
                const uint32_t i1 = std::min(n, i0 + grain);
                for (uint32_t i = i0; i < i1; ++i) f(i, t);
            }
        });
    for (auto& th : pool) th.join();
}

// The full operator build state (the members of Operator used during
// CalcECOperator).
// Effective material of the edges inside one UPML slab, kept from the EC
// pass for the UPML build (which needs the same AverageMatQuarterCell values:
// eff[0], eff[1], eff[2] per edge direction), so it is evaluated once.
struct SlabEff {
    uint32_t start[3], nl[3];
    std::vector<double> v;  // [3 directions][nl0][nl1][nl2][3]
    bool holds(const uint32_t* pos) const {
        for (int a = 0; a < 3; ++a)
            if (pos[a] < start[a] || pos[a] >= start[a] + nl[a]) return false;
        return true;
    }
    size_t at(int n, const uint32_t* pos) const {
        const size_t nloc = (size_t)nl[0] * nl[1] * nl[2];
        const size_t li = ((size_t)(pos[0] - start[0]) * nl[1] + (pos[1] - start[1])) * nl[2] + (pos[2] - start[2]);
        return 3 * ((size_t)n * nloc + li);
    }
};

struct Builder {
    const fdtd_scene_s& S;
    Geo g;
    uint32_t N[3];
    size_t NN;
    int threads;
    BoxIndex mat_idx, pec_idx, exc_idx;
    std::vector<float> EC_C, EC_G, EC_L, EC_R;  // [3][N]  (operator.h:267-270)
    std::vector<float> vv, vi, ii, iv;          // [3][N]
    double dT = 0;
    int BC[6];
    uint32_t pml[6];

    explicit Builder(const fdtd_scene_s& s, int nthreads) : S(s), threads(nthreads) {
        for (int n = 0; n < 3; ++n) N[n] = (uint32_t)s.lines[n].size();
        g.L = s.lines;
        for (int n = 0; n < 3; ++n) g.N[n] = N[n];
        g.unit = s.unit;
        g.cache();
        NN = (size_t)N[0] * N[1] * N[2];
        for (int i = 0; i < 6; ++i) {
            BC[i] = s.bc[i];
            pml[i] = s.pml_size[i];
        }
    }
    size_t at(int n, uint32_t x, uint32_t y, uint32_t z) const {
        return (size_t)n * NN + ((size_t)x * N[1] + y) * N[2] + z;
    }
    size_t at(int n, const uint32_t* p) const { return at(n, p[0], p[1], p[2]); }

    // Operator::AverageMatQuarterCell (operator.cpp:1406-1518) and
    // Operator::Calc_ECPos (operator.cpp:1176-1224) for the edges in
    // direction ny along one z-line (x, y), every z at once.
    //
    // GetMaterial's box lookup: the winner for a sample is the first set bit
    // of the three per-axis masks ANDed (BoxIndex::lookup); the x and y
    // masks of the six samples are fixed along the line, so they are ANDed
    // once per line.  The geometry comes from per-axis tables of the same
    // products the reference forms (GetNodeWidth / GetEdgeLength =
    // disc delta * unit; GetNodeArea = the product of two widths, 0 when a
    // shifted position is negative).  Every product, sum and quotient is
    // then formed in the reference's order, so the values are identical.
    struct EcLine {
        // Wm[a][i]: GetNodeWidth(a, i, dual) = GetEdgeLength(a, i, main);
        // Dm[a][i]: GetNodeWidth(a, i, main) = GetEdgeLength(a, i, dual)
        std::vector<double> Wm[3], Dm[3];
        // material table indexed by winner bit; the last entry is the background
        std::vector<double> eps, kappa, mue, sigma;
    };
    EcLine ec_tables() const {
        EcLine t;
        for (int a = 0; a < 3; ++a) {
            t.Wm[a].resize(N[a]);
            t.Dm[a].resize(N[a]);
            for (uint32_t i = 0; i < N[a]; ++i) {
                t.Wm[a][i] = g.disc_delta(a, i, false) * g.unit;
                t.Dm[a][i] = g.disc_delta(a, i, true) * g.unit;
            }
        }
        const size_t nb = mat_idx.prim.size();
        t.eps.resize(nb + 1); t.kappa.resize(nb + 1); t.mue.resize(nb + 1); t.sigma.resize(nb + 1);
        for (size_t b = 0; b < nb; ++b) {
            const Prim& p = S.prims[mat_idx.prim[b]];
            t.eps[b] = p.eps; t.kappa[b] = p.kappa; t.mue[b] = p.mue; t.sigma[b] = p.sigma;
        }
        t.eps[nb] = S.bg_eps; t.kappa[nb] = S.bg_kappa; t.mue[nb] = S.bg_mue; t.sigma[nb] = S.bg_sigma;
        return t;
    }

    // The edges (ny, x, y, z) for every z: EC[4][z] and EffMat[3][z] (eps,
    // kappa, mue averages) into ec / eff; false when an effective material
    // parameter is NaN or Inf.  m01: scratch of 6 * W words.
    bool ec_line(const EcLine& t, int ny, uint32_t x, uint32_t y, double* ec, double* eff,
                 std::vector<uint64_t>& m01) const {
        const int n = ny, nP = (n + 1) % 3, nPP = (n + 2) % 3;
        const int W = mat_idx.W;
        const size_t nb = mat_idx.prim.size();
        // sample kinds per axis of the six lookups: the four quarter cells
        // (up-right, up-left, down-right, down-left), then the two half
        // lines below and above the node along ny
        int kind[6][3];
        const int qP[4] = {SK_QP, SK_QM, SK_QP, SK_QM}, qPP[4] = {SK_QP, SK_QP, SK_QM, SK_QM};
        for (int q = 0; q < 4; ++q) {
            kind[q][n] = SK_HALF;
            kind[q][nP] = qP[q];
            kind[q][nPP] = qPP[q];
        }
        for (int q = 4; q < 6; ++q) {
            kind[q][n] = q == 4 ? SK_QM : SK_QP;
            kind[q][nP] = SK_HALF;
            kind[q][nPP] = SK_HALF;
        }
        m01.resize(6 * (size_t)W);
        if (nb)
            for (int q = 0; q < 6; ++q) {
                const uint64_t* a0 = &mat_idx.masks[0][kind[q][0]][(size_t)x * W];
                const uint64_t* a1 = &mat_idx.masks[1][kind[q][1]][(size_t)y * W];
                for (int w = 0; w < W; ++w) m01[q * W + w] = a0[w] & a1[w];
            }
        auto winner = [&](int q, uint32_t z) -> size_t {
            if (!nb) return nb;
            const uint64_t* a2 = &mat_idx.masks[2][kind[q][2]][(size_t)z * W];
            for (int w = 0; w < W; ++w) {
                const uint64_t m = m01[q * W + w] & a2[w];
                if (m) return (size_t)w * 64 + (size_t)__builtin_ctzll(m);
            }
            return nb;
        };
        const uint32_t pos_xy[2] = {x, y};
        bool ok = true;
        for (uint32_t z = 0; z < N[2]; ++z) {
            const uint32_t pos[3] = {pos_xy[0], pos_xy[1], z};
            const uint32_t p = pos[nP], pp = pos[nPP], pn = pos[n];
            // quarter-cell areas GetNodeArea(ny, loc, dual) of the four shifts
            const double wP0 = t.Wm[nP][p], wPP0 = t.Wm[nPP][pp];
            const double wP1 = p ? t.Wm[nP][p - 1] : 0, wPP1 = pp ? t.Wm[nPP][pp - 1] : 0;
            const double A[4] = {wP0 * wPP0, p ? wP1 * wPP0 : 0.0, pp ? wP0 * wPP1 : 0.0,
                                 (p && pp) ? wP1 * wPP1 : 0.0};
            double E0, E1, area = 0;
            {
                size_t w = winner(0, z);
                E0 = t.eps[w] * A[0];
                E1 = t.kappa[w] * A[0];
                area += A[0];
                for (int q = 1; q < 4; ++q) {
                    w = winner(q, z);
                    E0 += t.eps[w] * A[q];
                    E1 += t.kappa[w] * A[q];
                    area += A[q];
                }
            }
            E0 *= kEps0 / area;
            E1 /= area;
            // mu, sigma: harmonic along ny over the half lines below and above
            double E2, E3, length;
            {
                double delta_ny = pn ? t.Wm[n][pn - 1] : 0;
                size_t w = winner(4, z);
                E2 = delta_ny / t.mue[w];
                double sigma = t.sigma[w];
                E3 = sigma ? delta_ny / sigma : 0;
                length = delta_ny;
                delta_ny = t.Wm[n][pn];
                w = winner(5, z);
                E2 += delta_ny / t.mue[w];
                sigma = t.sigma[w];
                if (sigma)
                    E3 += delta_ny / sigma;
                else
                    E3 = 0;
                length += delta_ny;
            }
            E2 = length * kMue0 / E2;
            if (E3) E3 = length / E3;
            if (std::isnan(E0) || std::isinf(E0) || std::isnan(E1) || std::isinf(E1) || std::isnan(E2) ||
                std::isinf(E2) || std::isnan(E3) || std::isinf(E3)) {
                ok = false;
                break;
            }
            // Calc_ECPos
            double delta = t.Wm[n][pn];
            double ar = t.Dm[nP][p] * t.Dm[nPP][pp];
            double* e = ec + 4 * (size_t)z;
            if (delta) {
                e[0] = E0 * ar / delta;
                e[1] = E1 * ar / delta;
            } else {
                e[0] = 0;
                e[1] = 0;
            }
            delta = t.Dm[n][pn];
            ar = t.Wm[nP][p] * t.Wm[nPP][pp];
            if (delta) {
                e[2] = E2 * ar / delta;
                e[3] = E3 * ar / delta;
            } else {
                e[2] = 0;
                e[3] = 0;
            }
            double* f = eff + 3 * (size_t)z;
            f[0] = E0;
            f[1] = E1;
            f[2] = E2;
        }
        return ok;
    }

    // Operator::Calc_EC_Range over all lines; the effective materials of
    // edges inside the given UPML slabs are kept in them (slabs do not overlap)
    bool calc_ec(std::vector<SlabEff>* slabs = nullptr) {
        EC_C.assign(3 * NN, 0.f);
        EC_G.assign(3 * NN, 0.f);
        EC_L.assign(3 * NN, 0.f);
        EC_R.assign(3 * NN, 0.f);
        if (slabs)
            for (SlabEff& se : *slabs) se.v.assign(9 * (size_t)se.nl[0] * se.nl[1] * se.nl[2], 0.0);
        const EcLine t = ec_tables();
        std::atomic<bool> ok{true};
        parallel_for(N[0], threads, [&](uint32_t x, int) {
            std::vector<double> ec(4 * (size_t)N[2]), eff(3 * (size_t)N[2]);
            std::vector<uint64_t> m01;
            for (uint32_t y = 0; y < N[1]; ++y)
                for (int n = 0; n < 3; ++n) {
                    if (!ec_line(t, n, x, y, ec.data(), eff.data(), m01)) {
                        ok = false;
                        return;
                    }
                    const size_t i0 = at(n, x, y, 0);
                    for (uint32_t z = 0; z < N[2]; ++z) {
                        EC_C[i0 + z] = (float)ec[4 * z];
                        EC_G[i0 + z] = (float)ec[4 * z + 1];
                        EC_L[i0 + z] = (float)ec[4 * z + 2];
                        EC_R[i0 + z] = (float)ec[4 * z + 3];
                    }
                    if (slabs)
                        for (SlabEff& se : *slabs) {
                            uint32_t pos[3] = {x, y, se.start[2]};
                            if (!se.holds(pos)) continue;
                            for (uint32_t z = se.start[2]; z < se.start[2] + se.nl[2]; ++z) {
                                pos[2] = z;
                                double* d = &se.v[se.at(n, pos)];
                                d[0] = eff[3 * z];
                                d[1] = eff[3 * z + 1];
                                d[2] = eff[3 * z + 2];
                            }
                        }
                }
        });
        if (!ok) set_error("an effective material parameter is NaN or Inf (AverageMatQuarterCell)");
        return ok;
    }

    // AdrOp::GetPos with SetReflection2Cell (tools/AdrOp.cpp:183-221, 429-433)
    static uint32_t refl(int q, uint32_t M) {
        if (q < 0) return (uint32_t)(-q - 1);
        if (q > (int)M - 1) return (uint32_t)(2 * ((int)M - 1) - q + 1);
        return (uint32_t)q;
    }
    size_t shifted(int n, const uint32_t* pos, const int* sh) const {
        uint32_t p[3];
        for (int a = 0; a < 3; ++a) p[a] = refl((int)pos[a] + sh[a], N[a]);
        return at(n, p);
    }

    // Operator::CalcTimestep_Var3 (operator.cpp:1897-1971).  The terms are
    // evaluated as the reference does: float products / reciprocals of the
    // float EC arrays, accumulated into doubles.
    double node_dt_var3(int n, const uint32_t* pos) const {
        int nP = (n + 1) % 3, nPP = (n + 2) % 3;
        int s0[3] = {0, 0, 0};
        int sP1[3] = {0, 0, 0}; sP1[nP] = 1;
        int sPP1[3] = {0, 0, 0}; sPP1[nPP] = 1;
        int sPm[3] = {0, 0, 0}; sPm[nP] = -1;
        int sPPm[3] = {0, 0, 0}; sPPm[nPP] = -1;
        int sPmPPm[3] = {0, 0, 0}; sPmPPm[nP] = -1; sPmPPm[nPP] = -1;
        int sN1[3] = {0, 0, 0}; sN1[n] = 1;
        auto C = [&](int c, const int* s) { return EC_C[(size_t)c * NN + shifted(0, pos, s)]; };
        auto Lf = [&](int c, const int* s) { return EC_L[(size_t)c * NN + shifted(0, pos, s)]; };
        float one = 1;
        double wqp = one / (Lf(nPP, s0) * C(n, sP1)) + one / (Lf(nPP, s0) * C(n, s0));
        wqp += one / (Lf(nP, s0) * C(n, sPP1)) + one / (Lf(nP, s0) * C(n, s0));
        // ipos = Shift(nP,-1); GetShiftedPos(nP,1) == pos
        wqp += one / (Lf(nPP, sPm) * C(n, s0)) + one / (Lf(nPP, sPm) * C(n, sPm));
        // ipos = Shift(nPP,-1) (shift nP and nPP by -1); GetShiftedPos(nPP,1) -> nP-1 only
        wqp += one / (Lf(nP, sPmPPm) * C(n, sPm)) + one / (Lf(nP, sPmPPm) * C(n, sPmPPm));

        double wt_4[4];
        wt_4[0] = one / (Lf(nPP, s0) * C(nP, s0));
        wt_4[1] = one / (Lf(nPP, sPm) * C(nP, s0));
        wt_4[2] = one / (Lf(nP, s0) * C(nPP, s0));
        wt_4[3] = one / (Lf(nP, sPPm) * C(nPP, s0));
        double wt1 = wt_4[0] + wt_4[1] + wt_4[2] + wt_4[3] - 2 * min4(wt_4);

        wt_4[0] = one / (Lf(nPP, s0) * C(nP, sN1));
        wt_4[1] = one / (Lf(nPP, sPm) * C(nP, sN1));
        wt_4[2] = one / (Lf(nP, s0) * C(nPP, sN1));
        wt_4[3] = one / (Lf(nP, sPPm) * C(nPP, sN1));
        double wt2 = wt_4[0] + wt_4[1] + wt_4[2] + wt_4[3] - 2 * min4(wt_4);

        double w_total = wqp + wt1 + wt2;
        return 2 / std::sqrt(w_total);
    }

    // The same terms for the interior run z in [1, N2-2] of the line (x, y)
    // (x, y interior): every shift stays on the grid, so each operand is a
    // fixed offset from the line and the loop runs over z with plain pointer
    // reads (the compiler vectorizes it; every operation is the scalar one,
    // in the same order, so the values are identical).
    void line_dt_var3(int n, uint32_t x, uint32_t y, double* out) const {
        const int nP = (n + 1) % 3, nPP = (n + 2) % 3;
        const long long st[3] = {(long long)N[1] * N[2], (long long)N[2], 1};
        const float* Lb = EC_L.data() + at(0, x, y, 0);
        const float* Cb = EC_C.data() + at(0, x, y, 0);
        const long long cn = (long long)n * NN, cp = (long long)nP * NN, cpp = (long long)nPP * NN;
        const float* Lpp_0 = Lb + cpp;
        const float* Lp_0 = Lb + cp;
        const float* Lpp_m = Lb + cpp - st[nP];
        const float* Lp_mm = Lb + cp - st[nP] - st[nPP];
        const float* Lp_ppm = Lb + cp - st[nPP];
        const float* Cn_0 = Cb + cn;
        const float* Cn_p1 = Cb + cn + st[nP];
        const float* Cn_pp1 = Cb + cn + st[nPP];
        const float* Cn_m = Cb + cn - st[nP];
        const float* Cn_mm = Cb + cn - st[nP] - st[nPP];
        const float* Cp_0 = Cb + cp;
        const float* Cpp_0 = Cb + cpp;
        const float* Cp_n1 = Cb + cp + st[n];
        const float* Cpp_n1 = Cb + cpp + st[n];
        const float one = 1;
        const uint32_t z1 = N[2] - 1;
        for (uint32_t z = 1; z < z1; ++z) {
            double wqp = one / (Lpp_0[z] * Cn_p1[z]) + one / (Lpp_0[z] * Cn_0[z]);
            wqp += one / (Lp_0[z] * Cn_pp1[z]) + one / (Lp_0[z] * Cn_0[z]);
            wqp += one / (Lpp_m[z] * Cn_0[z]) + one / (Lpp_m[z] * Cn_m[z]);
            wqp += one / (Lp_mm[z] * Cn_m[z]) + one / (Lp_mm[z] * Cn_mm[z]);
            double a0 = one / (Lpp_0[z] * Cp_0[z]), a1 = one / (Lpp_m[z] * Cp_0[z]);
            double a2 = one / (Lp_0[z] * Cpp_0[z]), a3 = one / (Lp_ppm[z] * Cpp_0[z]);
            double m = a0;
            m = a1 < m ? a1 : m;
            m = a2 < m ? a2 : m;
            m = a3 < m ? a3 : m;
            const double wt1 = a0 + a1 + a2 + a3 - 2 * m;
            a0 = one / (Lpp_0[z] * Cp_n1[z]);
            a1 = one / (Lpp_m[z] * Cp_n1[z]);
            a2 = one / (Lp_0[z] * Cpp_n1[z]);
            a3 = one / (Lp_ppm[z] * Cpp_n1[z]);
            m = a0;
            m = a1 < m ? a1 : m;
            m = a2 < m ? a2 : m;
            m = a3 < m ? a3 : m;
            const double wt2 = a0 + a1 + a2 + a3 - 2 * m;
            const double w_total = wqp + wt1 + wt2;
            out[z] = 2 / std::sqrt(w_total);
        }
    }

    double calc_timestep_var3() const {
        std::vector<double> best(std::max(threads, 1), 1e200);
        parallel_for(N[0], threads, [&](uint32_t x, int t) {
            uint32_t pos[3] = {x, 0, 0};
            double dT_loc = best[t];
            std::vector<double> line(N[2]);
            auto take = [&](double newT) {
                if ((newT < dT_loc) && (newT > 0.0)) dT_loc = newT;
            };
            // (the minimum does not depend on the visiting order)
            for (int n = 0; n < 3; ++n)
                for (pos[1] = 0; pos[1] < N[1]; ++pos[1]) {
                    const bool fast = x > 0 && x + 1 < N[0] && pos[1] > 0 && pos[1] + 1 < N[1] && N[2] > 2;
                    if (fast) {
                        line_dt_var3(n, x, pos[1], line.data());
                        for (uint32_t z = 1; z + 1 < N[2]; ++z) take(line[z]);
                        pos[2] = 0;
                        take(node_dt_var3(n, pos));
                        pos[2] = N[2] - 1;
                        take(node_dt_var3(n, pos));
                    } else {
                        for (pos[2] = 0; pos[2] < N[2]; ++pos[2]) take(node_dt_var3(n, pos));
                    }
                }
            best[t] = dT_loc;
        });
        double r = 1e200;
        for (double b : best) r = std::min(r, b);
        return r;
    }
    static double min4(const double* v) {  // min(double*, count) (operator.cpp:1886-1895)
        double m = v[0];
        for (int k = 1; k < 4; ++k)
            if (v[k] < m) m = v[k];
        return m;
    }

    // Operator::Calc_ECOperatorPos (operator.cpp:943-971)
    void ec_operator_pos(int n, const uint32_t* pos) {
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

    void apply_electric_bc(const bool* dirs) {  // operator.cpp:1086-1129
        uint32_t pos[3];
        for (int n = 0; n < 3; ++n) {
            int nP = (n + 1) % 3, nPP = (n + 2) % 3;
            for (pos[nP] = 0; pos[nP] < N[nP]; ++pos[nP])
                for (pos[nPP] = 0; pos[nPP] < N[nPP]; ++pos[nPP]) {
                    if (dirs[2 * n]) {
                        pos[n] = 0;
                        vv[at(nP, pos)] = 0; vi[at(nP, pos)] = 0;
                        vv[at(nPP, pos)] = 0; vi[at(nPP, pos)] = 0;
                    }
                    if (dirs[2 * n + 1]) {
                        pos[n] = N[n] - 1;
                        vv[at(n, pos)] = 0; vi[at(n, pos)] = 0;
                        vv[at(nP, pos)] = 0; vi[at(nP, pos)] = 0;
                        vv[at(nPP, pos)] = 0; vi[at(nPP, pos)] = 0;
                    }
                }
        }
    }

    void apply_magnetic_bc(const bool* dirs) {  // operator.cpp:1131-1174
        uint32_t pos[3];
        for (int n = 0; n < 3; ++n) {
            int nP = (n + 1) % 3, nPP = (n + 2) % 3;
            for (pos[nP] = 0; pos[nP] < N[nP]; ++pos[nP])
                for (pos[nPP] = 0; pos[nPP] < N[nPP]; ++pos[nPP]) {
                    if (dirs[2 * n]) {
                        pos[n] = 0;
                        for (int c : {n, nP, nPP}) { ii[at(c, pos)] = 0; iv[at(c, pos)] = 0; }
                    }
                    if (dirs[2 * n + 1]) {
                        pos[n] = N[n] - 2;
                        for (int c : {nP, nPP}) { ii[at(c, pos)] = 0; iv[at(c, pos)] = 0; }
                    }
                    pos[n] = N[n] - 1;
                    for (int c : {n, nP, nPP}) { ii[at(c, pos)] = 0; iv[at(c, pos)] = 0; }
                }
        }
    }

    void calc_pec() {  // CalcPEC_Range (operator.cpp:1986-2020); no curves in the box model
        parallel_for(N[0], threads, [&](uint32_t x, int) {
            uint32_t pos[3] = {x, 0, 0};
            for (pos[1] = 0; pos[1] < N[1]; ++pos[1])
                for (pos[2] = 0; pos[2] < N[2]; ++pos[2])
                    for (int n = 0; n < 3; ++n) {
                        int kind[3] = {SK_LINE, SK_LINE, SK_LINE};
                        kind[n] = SK_DUAL;
                        int w = pec_idx.lookup(kind, pos);
                        if (w >= 0 && S.prims[w].kind == PK_METAL) {
                            vv[at(n, pos)] = 0;
                            vi[at(n, pos)] = 0;
                        }
                    }
        });
    }

    bool calc_lumped() {  // Operator::Calc_LumpedElements (operator.cpp:1535-1712)
        for (const Prim& p : S.prims) {
            if (p.kind != PK_LUMPED) continue;
            // only parallel R/C elements (IsLEparRC, operator.cpp:1714-1724);
            // the rest belong to the lumped RLC extension
            if (!(p.le_type == FDTD_LE_PARALLEL && !(p.L > 0))) continue;
            double C = p.C;
            if (C <= 0) C = NAN;
            double R = p.R;
            if (R < 0) R = NAN;
            if (std::isnan(R) && std::isnan(C)) continue;
            int ny = p.ny;
            if (ny < 0 || ny > 2) continue;
            int nyP = (ny + 1) % 3, nyPP = (ny + 2) % 3;
            uint32_t uiStart[3], uiStop[3];
            int dim = g.snap_box(p.start, p.stop, uiStart, uiStop, false, 0, nullptr, nullptr);
            if (dim <= 0) continue;
            if (uiStart[ny] == uiStop[ny]) continue;
            uint32_t pos[3];
            double unitGC = 0;
            for (pos[ny] = uiStart[ny]; pos[ny] < uiStop[ny]; ++pos[ny]) {
                double plane = 0;
                for (pos[nyP] = uiStart[nyP]; pos[nyP] <= uiStop[nyP]; ++pos[nyP])
                    for (pos[nyPP] = uiStart[nyPP]; pos[nyPP] <= uiStop[nyPP]; ++pos[nyPP])
                        plane += g.edge_area(ny, pos, false) / g.edge_length(ny, pos, false);
                unitGC += 1 / plane;
            }
            unitGC = 1 / unitGC;
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
                        if (C > 0) EC_C[i] = (float)(epsilon * g.edge_area(ny, pos, false) / g.edge_length(ny, pos, false));
                        if (R > 0) EC_G[i] = (float)(kappa * g.edge_area(ny, pos, false) / g.edge_length(ny, pos, false));
                        if (R == 0) {
                            vv[i] = 0;
                            vi[i] = 0;
                        } else
                            ec_operator_pos(ny, pos);
                    }
            if (p.caps) {
                for (pos[nyP] = uiStart[nyP]; pos[nyP] <= uiStop[nyP]; ++pos[nyP])
                    for (pos[nyPP] = uiStart[nyPP]; pos[nyPP] <= uiStop[nyPP]; ++pos[nyPP]) {
                        for (uint32_t end : {uiStart[ny], uiStop[ny]}) {
                            pos[ny] = end;
                            if (pos[nyP] < uiStop[nyP]) { vv[at(nyP, pos)] = 0; vi[at(nyP, pos)] = 0; }
                            if (pos[nyPP] < uiStop[nyPP]) { vv[at(nyPP, pos)] = 0; vi[at(nyPP, pos)] = 0; }
                        }
                    }
            }
        }
        return true;
    }

    // Operator_Ext_LumpedRLC::BuildExtension (operator_ext_lumpedRLC.cpp:
    // 112-486): parallel R||L||C and series R-L-C elements.  Each box is
    // split into Ncells_0 edges in series along its direction and
    // Ncells_1 x Ncells_2 in parallel across it; the element's R, L, C are
    // scaled accordingly.  The edge's own capacitance carries C (parallel)
    // or stays the parasitic capacitance, raised where it would short the
    // element below fmax (series, and parallel without C); G is replaced;
    // vv/vi (and ii/iv) of the edge are recomputed from EC_C/EC_G/EC_L/EC_R.
    // The double coefficients are stored as float, as the reference copies
    // its double vectors into FDTD_FLOAT arrays.
    void calc_rlc(double fmax, RlcList& out) {
        constexpr double kZFact = 20.0;  // LUMPED_RLC_Z_FACT (operator_ext_lumpedRLC.h:29)
        for (const Prim& p : S.prims) {
            if (p.kind != PK_LUMPED) continue;
            const int type = p.le_type;
            double C = p.C;
            if (C < 0) C = NAN;
            double R = p.R;
            if (R < 0) R = NAN;
            double L = p.L;
            if (L < 0) L = NAN;
            // IsLElumpedRLC (operator_ext_lumpedRLC.cpp:502-513)
            if (!((type == FDTD_LE_PARALLEL && L > 0.0) || type == FDTD_LE_SERIES)) continue;
            const int dir = p.ny;
            if (dir < 0 || dir > 2) continue;
            const int d1 = (dir + 1) % 3, d2 = (dir + 2) % 3;
            uint32_t uiStart[3], uiStop[3];
            const int dim = g.snap_box(p.start, p.stop, uiStart, uiStop, false, 0, nullptr, nullptr);
            if (dim <= 0) continue;
            if (uiStart[dir] == uiStop[dir]) continue;
            const unsigned Ncells_0 = uiStop[dir] - uiStart[dir];
            const unsigned Ncells_1 = uiStop[d1] - uiStart[d1] + 1;
            const unsigned Ncells_2 = uiStop[d2] - uiStart[d2] + 1;
            const unsigned Npar = Ncells_1 * Ncells_2;
            const double dL = L * Npar / Ncells_0;
            const double dR = R * Npar / Ncells_0;
            double dG = (1 / R) * Ncells_0 / Npar;
            double dC = C * Ncells_0 / Npar;  // mutable across the box's edges, as in the reference
            const double ib0 = 2.0 * dT * dC / (4.0 * dL * dC + 2.0 * dT * dR * dC + dT * dT);
            const double b1 = (dT * dT - 4.0 * dL * dC) / (dT * dC);
            const double b2 = (4.0 * dL * dC - 2.0 * dT * dR * dC + dT * dT) / (2.0 * dT * dC);
            if (type == FDTD_LE_PARALLEL && R == 0.0) dG = 0.0;
            uint32_t pos[3];
            for (pos[dir] = uiStart[dir]; pos[dir] < uiStop[dir]; ++pos[dir])
                for (pos[d1] = uiStart[d1]; pos[d1] <= uiStop[d1]; ++pos[d1])
                    for (pos[d2] = uiStart[d2]; pos[d2] <= uiStop[d2]; ++pos[d2]) {
                        const size_t i = at(dir, pos);
                        double Zmin, Zcd_min;
                        if (type == FDTD_LE_PARALLEL) {
                            if (dC > 0)
                                EC_C[i] = (float)dC;
                            else
                                dC = EC_C[i];
                            out.i2v.push_back((float)((dT / dC) / (1.0 + dT * dG / (2.0 * dC))));
                            if (R >= 0) EC_G[i] = (float)dG;
                            out.ilv.push_back(L > 0 ? (float)(dT / dL) : 0.f);
                            if (dC == 0) {
                                double Cd = EC_C[i];
                                Zmin = std::max(dR, 2 * kPi * fmax * dL);
                                Zcd_min = 1.0 / (2.0 * kPi * fmax * Cd);
                                if (Zcd_min < kZFact * Zmin) {
                                    Cd = 1.0 / (2 * kPi * fmax * Zmin * kZFact);
                                    EC_C[i] = (float)Cd;
                                }
                            }
                            out.vv2.push_back(0.f);
                            out.vj1.push_back(0.f);
                            out.vj2.push_back(0.f);
                            out.vvd.push_back(1.f);
                            out.ib0.push_back(0.f);
                            out.b1.push_back(0.f);
                            out.b2.push_back(0.f);
                        } else {
                            EC_G[i] = 0.f;
                            float Cd = EC_C[i];  // FDTD_FLOAT in the reference
                            Zmin = std::sqrt(std::pow(dR, 2) + std::pow(2 * kPi * fmax * dL - 1.0 / (dC * 2 * kPi * fmax), 2));
                            Zcd_min = 1.0 / (2.0 * kPi * fmax * Cd);
                            if (Zcd_min < kZFact * Zmin) {
                                Cd = (float)(1.0 / (2 * kPi * fmax * Zmin * kZFact));
                                EC_C[i] = Cd;
                            }
                            out.ilv.push_back(0.f);
                            out.i2v.push_back(0.f);
                            out.vv2.push_back((float)(0.5 * dT * ib0 / Cd));
                            out.vj1.push_back((float)(0.5 * dT * (b1 * ib0 - 1.0) / Cd));
                            out.vj2.push_back((float)(0.5 * dT * b2 * ib0 / Cd));
                            out.vvd.push_back((float)(1.0 / (1.0 + 0.5 * dT * ib0 / Cd)));
                            out.ib0.push_back((float)ib0);
                            out.b1.push_back((float)b1);
                            out.b2.push_back((float)b2);
                        }
                        ec_operator_pos(dir, pos);
                        out.dir.push_back(dir);
                        for (int a = 0; a < 3; ++a) out.pos[a].push_back(pos[a]);
                    }
            if (p.caps) {  // metal caps at both ends, as Calc_LumpedElements builds them
                for (pos[d1] = uiStart[d1]; pos[d1] <= uiStop[d1]; ++pos[d1])
                    for (pos[d2] = uiStart[d2]; pos[d2] <= uiStop[d2]; ++pos[d2])
                        for (uint32_t end : {uiStart[dir], uiStop[dir]}) {
                            pos[dir] = end;
                            if (pos[d1] < uiStop[d1]) { vv[at(d1, pos)] = 0; vi[at(d1, pos)] = 0; }
                            if (pos[d2] < uiStop[d2]) { vv[at(d2, pos)] = 0; vi[at(d2, pos)] = 0; }
                        }
            }
        }
    }
};

// ---------------------------------------------------------------- UPML
// default grading function (operator_ext_upml.cpp:31):
//   -log(1e-6)*log(2.5)/(2*dl*Z*(pow(2.5,W/dl)-1)) * pow(2.5, D/dl)
double upml_grading(double D, double dl, double W, double Z) {
    return -std::log(1e-6) * std::log(2.5) / (2 * dl * Z * (std::pow(2.5, W / dl) - 1)) * std::pow(2.5, D / dl);
}

struct UpmlBuild {
    int BC[6];
    uint32_t Size[6];
    uint32_t start[3], nl[3];
};

// Operator_Ext_UPML::CalcGradingKappa (operator_ext_upml.cpp:289-363)
void grading_kappa(const Geo& g, const UpmlBuild& u, int ny, const uint32_t* pos, double Zm,
                   double* kv, double* ki) {
    double depth = 0, width = 0;
    for (int n = 0; n < 3; ++n) {
        if ((pos[n] <= u.Size[2 * n]) && (u.BC[2 * n] == 3)) {
            width = (g.line(n, u.Size[2 * n], false) - g.line(n, 0, false)) * g.unit;
            depth = width - (g.line(n, pos[n], false) - g.line(n, 0, false)) * g.unit;
            if (n == ny) depth -= g.edge_length(n, pos, false) / 2;
            double D = depth, dl = width / u.Size[2 * n], W = width;
            kv[n] = (depth > 0) ? upml_grading(D, dl, W, Zm) : 0;
            if (n == ny) depth += g.edge_length(n, pos, false) / 2;
            if (n != ny) depth -= g.edge_length(n, pos, false) / 2;
            if (depth < 0) depth = 0;
            ki[n] = (depth > 0) ? upml_grading(depth, dl, W, Zm) : 0;
        } else if ((pos[n] >= g.N[n] - 1 - u.Size[2 * n + 1]) && (u.BC[2 * n + 1] == 3)) {
            width = (g.line(n, g.N[n] - 1, false) - g.line(n, g.N[n] - u.Size[2 * n + 1] - 1, false)) * g.unit;
            depth = width - (g.line(n, g.N[n] - 1, false) - g.line(n, pos[n], false)) * g.unit;
            if (n == ny) depth += g.edge_length(n, pos, false) / 2;
            // the reference divides by the lower-side size here as well
            double dl = width / (u.Size[2 * n]), W = width;
            kv[n] = (depth > 0) ? upml_grading(depth, dl, W, Zm) : 0;
            if (n == ny) depth -= g.edge_length(n, pos, false) / 2;
            if (n != ny) depth += g.edge_length(n, pos, false) / 2;
            if (depth > width) depth = 0;
            ki[n] = (depth > 0) ? upml_grading(depth, dl, W, Zm) : 0;
        } else {
            kv[n] = 0;
            ki[n] = 0;
        }
    }
}

// Operator_Ext_UPML::Create_UPML slab ranges (operator_ext_upml.cpp:77-201)
std::vector<UpmlBuild> create_upml(const uint32_t* N, const int* ui_BC, const uint32_t* ui_size) {
    int BC[6];
    uint32_t size[6];
    for (int i = 0; i < 6; ++i) {
        BC[i] = ui_BC[i];
        size[i] = ui_size[i];
    }
    for (int n = 0; n < 3; ++n)
        if ((size[2 * n] * (BC[2 * n] == 3) + size[2 * n + 1] * (BC[2 * n + 1] == 3)) >= N[n]) {
            BC[2 * n] = 0; size[2 * n] = 0;
            BC[2 * n + 1] = 0; size[2 * n + 1] = 0;
        }
    std::vector<UpmlBuild> out;
    uint32_t start[3] = {0, 0, 0};
    uint32_t stop[3] = {N[0] - 1, N[1] - 1, N[2] - 1};
    auto add = [&]() {
        UpmlBuild u;
        for (int i = 0; i < 6; ++i) { u.BC[i] = BC[i]; u.Size[i] = size[i]; }
        for (int n = 0; n < 3; ++n) { u.start[n] = start[n]; u.nl[n] = stop[n] - start[n] + 1; }
        out.push_back(u);
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
    return out;
}

}  // namespace

void set_error(const std::string& msg) { g_last_error = msg; }
const std::string& last_error() { return g_last_error; }

// ------------------------------------------------------------ full build
static int build_operator(const fdtd_scene_s& S, int threads, fdtd_operator_s& op) {
    Builder B(S, threads);
    for (int n = 0; n < 3; ++n) {
        if (B.N[n] < 2) {
            set_error("every axis needs at least two mesh lines");
            return FDTD_ERR_ARG;
        }
    }
    B.mat_idx.build(S.prims, is_material, B.g);
    B.pec_idx.build(S.prims, is_mat_or_metal, B.g);
    B.exc_idx.build(S.prims, is_excitation, B.g);

    // the UPML slabs (operator_ext_upml.cpp:77-255) depend only on the grid and
    // the boundary settings; their edges' effective materials come out of the
    // EC pass
    std::vector<UpmlBuild> ub = create_upml(B.N, S.bc, S.pml_size);
    // openEMS computes the slab ranges in unsigned arithmetic
    // (operator_ext_upml.cpp:139-201): where an axis has fewer lines than its
    // two faces' sizes + 2 (a face that is not PML counts as 8 on x, the
    // y / z slabs ending size[0]+1 lines before the x-max face, :163), a
    // range ends before it starts and wraps around; such an operator cannot
    // be built
    for (const UpmlBuild& u : ub)
        for (int a = 0; a < 3; ++a)
            if (u.nl[a] == 0 || (uint64_t)u.start[a] + u.nl[a] > B.N[a]) {
                set_error("fdtd_operator_build: a UPML slab range leaves the grid (openEMS's ranges wrap around on an "
                          "axis with fewer lines than its faces' UPML sizes + 2; a face that is not PML counts as 8 "
                          "on x)");
                return FDTD_ERR_ARG;
            }
    std::vector<SlabEff> slab_eff(ub.size());
    for (size_t k = 0; k < ub.size(); ++k)
        for (int a = 0; a < 3; ++a) {
            slab_eff[k].start[a] = ub[k].start[a];
            slab_eff[k].nl[a] = ub[k].nl[a];
        }
    if (!B.calc_ec(&slab_eff)) return FDTD_ERR_ARG;

    // CalcTimestep (Var3, the default method 3, operator.cpp:52)
    B.dT = B.calc_timestep_var3();
    if (B.dT == 0 || B.dT >= 1e200) {
        set_error("timestep is zero: no valid edge found by CalcTimestep_Var3");
        return FDTD_ERR_ARG;
    }
    // m_TimeStepFactor = 1.  A periodic signal (the sinusoid) shortens dT
    // so that its period is a whole number of timesteps
    // (Operator::CalcECOperator, operator.cpp:1001-1007)
    if (S.have_excite && S.excite_type == 1) {
        const double period = 1 / S.f0;
        const unsigned int TS = (unsigned int)std::ceil(period / B.dT);
        B.dT = period / TS;
    }

    B.vv.assign(3 * B.NN, 0.f);
    B.vi.assign(3 * B.NN, 0.f);
    B.ii.assign(3 * B.NN, 0.f);
    B.iv.assign(3 * B.NN, 0.f);
    parallel_for(B.N[0], threads, [&](uint32_t x, int) {
        uint32_t pos[3] = {x, 0, 0};
        for (int n = 0; n < 3; ++n)
            for (pos[1] = 0; pos[1] < B.N[1]; ++pos[1])
                for (pos[2] = 0; pos[2] < B.N[2]; ++pos[2]) B.ec_operator_pos(n, pos);
    });

    bool PEC[6];
    for (int n = 0; n < 6; ++n) PEC[n] = S.bc[n] != -1;
    B.apply_electric_bc(PEC);
    B.calc_pec();
    B.calc_lumped();
    bool PMC[6];
    for (int n = 0; n < 6; ++n) PMC[n] = S.bc[n] == 1;
    B.apply_magnetic_bc(PMC);

    const Geo& g = B.g;
    const uint32_t* N = B.N;
    const double dT = B.dT;

    // ---- extension 1: excitation (operator_ext_excitation.cpp:101-285)
    // (only the index box in which some excitation primitive can match is
    // visited, in the reference's z, y, x order: the lookups outside it
    // return no primitive)
    uint32_t elo[3], ehi[3];
    const bool any_exc = B.exc_idx.span(0, elo[0], ehi[0]) && B.exc_idx.span(1, elo[1], ehi[1]) &&
                         B.exc_idx.span(2, elo[2], ehi[2]);
    if (any_exc) {
        uint32_t pos[3];
        for (pos[2] = elo[2]; pos[2] <= ehi[2]; ++pos[2])
            for (pos[1] = elo[1]; pos[1] <= ehi[1]; ++pos[1])
                for (pos[0] = elo[0]; pos[0] <= ehi[0]; ++pos[0]) {
                    double c[3];
                    for (int n = 0; n < 3; ++n) {
                        if (!g.yee_coords(n, pos, c, false)) continue;
                        int kind[3] = {SK_LINE, SK_LINE, SK_LINE};
                        kind[n] = SK_DUAL;
                        int w = B.exc_idx.lookup(kind, pos);
                        if (w < 0) continue;
                        const Prim& p = S.prims[w];
                        if (p.exc_type == 0 || p.exc_type == 1) {
                            double amp = p.exc_vec[n] * g.edge_length(n, pos, false);
                            if (amp != 0) {
                                op.volt_exc.amp.push_back((float)amp);
                                op.volt_exc.delay.push_back((uint32_t)(p.delay / dT));
                                op.volt_exc.dir.push_back((uint16_t)n);
                                for (int a = 0; a < 3; ++a) op.volt_exc.index[a].push_back(pos[a]);
                            }
                            if (p.exc_type == 1) {
                                B.vv[B.at(n, pos)] = 0;
                                B.vi[B.at(n, pos)] = 0;
                            }
                        }
                    }
                    for (int n = 0; n < 3; ++n) {
                        if ((pos[0] >= N[0] - 1) || (pos[1] >= N[1] - 1) || (pos[2] >= N[2] - 1)) continue;
                        if (!g.yee_coords(n, pos, c, true)) continue;
                        int kind[3] = {SK_DUAL, SK_DUAL, SK_DUAL};
                        kind[n] = SK_LINE;
                        int w = B.exc_idx.lookup(kind, pos);
                        if (w < 0) continue;
                        const Prim& p = S.prims[w];
                        if (p.exc_type == 2 || p.exc_type == 3) {
                            double amp = p.exc_vec[n] * g.edge_length(n, pos, true);
                            if (amp != 0) {
                                op.curr_exc.amp.push_back((float)amp);
                                op.curr_exc.delay.push_back((uint32_t)(p.delay / dT));
                                op.curr_exc.dir.push_back((uint16_t)n);
                                for (int a = 0; a < 3; ++a) op.curr_exc.index[a].push_back(pos[a]);
                            }
                            if (p.exc_type == 3) {
                                B.ii[B.at(n, pos)] = 0;
                                B.iv[B.at(n, pos)] = 0;
                            }
                        }
                    }
                }
    }

    // ---- extensions 2..7: UPML slabs (operator_ext_upml.cpp:365-466)
    // CalcGradingKappa's value on axis a depends only on (a, the line on a,
    // whether a is the edge direction) and on the boundary settings every
    // slab shares: tabulate it once per line with the same function, then
    // look it up per edge
    struct GradK {
        double kv, ki;
    };
    std::vector<GradK> gtab[3][2];
    if (!ub.empty()) {
        for (int a = 0; a < 3; ++a)
            for (int same = 0; same < 2; ++same) {
                gtab[a][same].resize(N[a]);
                parallel_for(N[a], threads, [&](uint32_t p, int) {
                    uint32_t pos[3] = {0, 0, 0};
                    pos[a] = p;
                    const int ny = same ? a : (a + 1) % 3;
                    double kv[3] = {0, 0, 0}, ki[3] = {0, 0, 0};
                    grading_kappa(g, ub[0], ny, pos, kZ0, kv, ki);
                    gtab[a][same][p] = GradK{kv[a], ki[a]};
                });
            }
    }
    for (size_t slab_k = 0; slab_k < ub.size(); ++slab_k) {
        const UpmlBuild& u = ub[slab_k];
        const SlabEff& se = slab_eff[slab_k];
        UpmlSlab slab;
        size_t nloc = (size_t)u.nl[0] * u.nl[1] * u.nl[2];
        for (int n = 0; n < 3; ++n) { slab.start[n] = u.start[n]; slab.num_lines[n] = u.nl[n]; }
        slab.vv.assign(3 * nloc, 0.f); slab.vvfo.assign(3 * nloc, 0.f); slab.vvfn.assign(3 * nloc, 0.f);
        slab.ii.assign(3 * nloc, 0.f); slab.iifo.assign(3 * nloc, 0.f); slab.iifn.assign(3 * nloc, 0.f);
        parallel_for(u.nl[0] * u.nl[1], threads, [&](uint32_t lxy, int) {
            uint32_t loc[3] = {lxy / u.nl[1], lxy % u.nl[1], 0};
            uint32_t pos[3];
            double kv[3] = {0, 0, 0}, ki[3] = {0, 0, 0}, eff[4];
            pos[0] = loc[0] + u.start[0];
            {
                pos[1] = loc[1] + u.start[1];
                for (loc[2] = 0; loc[2] < u.nl[2]; ++loc[2]) {
                    pos[2] = loc[2] + u.start[2];
                    for (int n = 0; n < 3; ++n) {
                        const double* ke = &se.v[se.at(n, pos)];  // AverageMatQuarterCell of the EC pass
                        eff[0] = ke[0];
                        eff[1] = ke[1];
                        eff[2] = ke[2];
                        for (int a = 0; a < 3; ++a) {  // grading_kappa(g, u, n, pos, kZ0, kv, ki)
                            const GradK& gk = gtab[a][a == n ? 1 : 0][pos[a]];
                            kv[a] = gk.kv;
                            ki[a] = gk.ki;
                        }
                        int nP = (n + 1) % 3, nPP = (n + 2) % 3;
                        size_t li = (size_t)n * nloc + ((size_t)loc[0] * u.nl[1] + loc[1]) * u.nl[2] + loc[2];
                        size_t gi = B.at(n, pos);
                        if (((kv[0] + kv[1] + kv[2]) != 0) && (eff[1] < 1e3)) {
                            if ((B.vv[gi] + B.vi[gi]) != 0) {
                                B.vv[gi] = (float)((2 * kEps0 - kv[nP] * dT) / (2 * kEps0 + kv[nP] * dT));
                                B.vi[gi] = (float)((2 * kEps0 * dT) / (2 * kEps0 + kv[nP] * dT) *
                                                   g.edge_length(n, pos, false) / g.edge_area(n, pos, false));
                                slab.vv[li] = (float)((2 * kEps0 - kv[nPP] * dT) / (2 * kEps0 + kv[nPP] * dT));
                                slab.vvfn[li] = (float)((2 * kEps0 + kv[n] * dT) / (2 * kEps0 + kv[nPP] * dT) / eff[0]);
                                slab.vvfo[li] = (float)((2 * kEps0 - kv[n] * dT) / (2 * kEps0 + kv[nPP] * dT) / eff[0]);
                            }
                        } else {
                            slab.vv[li] = B.vv[gi];
                            B.vv[gi] = 0;
                            slab.vvfo[li] = 0;
                            slab.vvfn[li] = 1;
                        }
                        if ((ki[0] + ki[1] + ki[2]) != 0) {
                            if ((B.ii[gi] + B.iv[gi]) != 0) {
                                B.ii[gi] = (float)((2 * kEps0 - ki[nP] * dT) / (2 * kEps0 + ki[nP] * dT));
                                B.iv[gi] = (float)((2 * kEps0 * dT) / (2 * kEps0 + ki[nP] * dT) *
                                                   g.edge_length(n, pos, true) / g.edge_area(n, pos, true));
                                slab.ii[li] = (float)((2 * kEps0 - ki[nPP] * dT) / (2 * kEps0 + ki[nPP] * dT));
                                slab.iifn[li] = (float)((2 * kEps0 + ki[n] * dT) / (2 * kEps0 + ki[nPP] * dT) / eff[2]);
                                slab.iifo[li] = (float)((2 * kEps0 - ki[n] * dT) / (2 * kEps0 + ki[nPP] * dT) / eff[2]);
                            }
                        } else {
                            slab.ii[li] = B.ii[gi];
                            B.ii[gi] = 0;
                            slab.iifo[li] = 0;
                            slab.iifn[li] = 1;
                        }
                    }
                }
            }
        }, std::max(1u, 4096u / std::max(1u, u.nl[2])));
        op.upml.push_back(std::move(slab));
    }

    // ---- extension 8: Lorentz / Drude (operator_ext_lorentzmaterial.cpp:117-438)
    int order = 0;
    bool have_lorentz = false;
    for (const Prim& p : S.prims)
        if (p.kind == PK_MATERIAL && p.lorentz) {
            have_lorentz = true;
            order = std::max(order, p.disp_order);
        }
    if (have_lorentz && order > 0) {
        for (int o = 0; o < order; ++o) {
            AdeOrder A;
            std::vector<double> v_int[3], v_ext[3], i_int[3], i_ext[3], v_lor[3], i_lor[3];
            uint32_t pos[3];
            for (pos[0] = 0; pos[0] < N[0]; ++pos[0])
                for (pos[1] = 0; pos[1] < N[1]; ++pos[1])
                    for (pos[2] = 0; pos[2] < N[2]; ++pos[2]) {
                        size_t index = ((size_t)pos[0] * N[1] + pos[1]) * N[2] + pos[2];
                        bool b_pos_on = false;
                        double L_D[3], R_D[3], C_L[3], C_D[3], G_D[3], L_L[3];
                        double c[3];
                        for (int n = 0; n < 3; ++n) {
                            L_D[n] = 0; R_D[n] = 0; C_L[n] = 0;
                            if (!g.yee_coords(n, pos, c, false)) continue;
                            if (B.vi[B.at(n, pos)] == 0) continue;
                            int kind[3] = {SK_LINE, SK_LINE, SK_LINE};
                            kind[n] = SK_DUAL;
                            int w = B.pec_idx.lookup(kind, pos);
                            if (w < 0) continue;
                            const Prim& p = S.prims[w];
                            if (p.kind == PK_MATERIAL && p.lorentz) {
                                double ecc = B.EC_C[(size_t)n * B.NN + index];
                                double w_plasma = (o < p.disp_order ? p.eps_plasma_f[o] : 0) * 2 * kPi;
                                if ((w_plasma > 0) && (ecc > 0)) {
                                    b_pos_on = true;
                                    A.volt_on = true;
                                    L_D[n] = 1 / (w_plasma * w_plasma * ecc);
                                }
                                double t_relax = (o < p.disp_order ? p.eps_relax_t[o] : 0);
                                if ((t_relax > 0) && A.volt_on) R_D[n] = L_D[n] / t_relax;
                                double w_lor = (o < p.disp_order ? p.eps_lor_pole_f[o] : 0) * 2 * kPi;
                                if ((w_lor > 0) && (L_D[n] > 0)) {
                                    A.volt_lor_on = true;
                                    C_L[n] = 1 / (w_lor * w_lor * L_D[n]);
                                }
                            }
                        }
                        // magnetic side: the same model on the dual edges, from
                        // the mue parameters and EC_L (lorentzmaterial.cpp:248-276)
                        for (int n = 0; n < 3; ++n) {
                            C_D[n] = 0; G_D[n] = 0; L_L[n] = 0;
                            if (!g.yee_coords(n, pos, c, true)) continue;
                            if (B.iv[B.at(n, pos)] == 0) continue;
                            int kind[3] = {SK_DUAL, SK_DUAL, SK_DUAL};
                            kind[n] = SK_LINE;
                            int w = B.pec_idx.lookup(kind, pos);
                            if (w < 0) continue;
                            const Prim& p = S.prims[w];
                            if (!(p.kind == PK_MATERIAL && p.lorentz)) continue;
                            double ecl = B.EC_L[(size_t)n * B.NN + index];
                            double w_plasma = (o < p.disp_order ? p.mue_plasma_f[o] : 0) * 2 * kPi;
                            if ((w_plasma > 0) && (ecl > 0)) {
                                b_pos_on = true;
                                A.curr_on = true;
                                C_D[n] = 1 / (w_plasma * w_plasma * ecl);
                            }
                            double t_relax = (o < p.disp_order ? p.mue_relax_t[o] : 0);
                            if ((t_relax > 0) && A.curr_on) G_D[n] = C_D[n] / t_relax;
                            double w_lor = (o < p.disp_order ? p.mue_lor_pole_f[o] : 0) * 2 * kPi;
                            if ((w_lor > 0) && (C_D[n] > 0)) {
                                A.curr_lor_on = true;
                                L_L[n] = 1 / (w_lor * w_lor * C_D[n]);
                            }
                        }
                        if (b_pos_on) {
                            for (int n = 0; n < 3; ++n) {
                                A.pos[n].push_back(pos[n]);
                                double viv = B.vi[B.at(n, pos)];
                                if (L_D[n] > 0) {
                                    v_int[n].push_back((2.0 * L_D[n] - dT * R_D[n]) / (2.0 * L_D[n] + dT * R_D[n]));
                                    v_ext[n].push_back(dT / (L_D[n] + dT * R_D[n] / 2.0) * viv);
                                } else if ((R_D[n] > 0) && (C_L[n] > 0)) {
                                    v_int[n].push_back((2.0 * dT - R_D[n] * C_L[n]) / (C_L[n] * R_D[n]));
                                    v_ext[n].push_back(2.0 / R_D[n] * viv);
                                } else {
                                    v_int[n].push_back(1);
                                    v_ext[n].push_back(0);
                                }
                                if (C_D[n] > 0) {
                                    double ivv = B.iv[B.at(n, pos)];
                                    i_int[n].push_back((2.0 * C_D[n] - dT * G_D[n]) / (2.0 * C_D[n] + dT * G_D[n]));
                                    i_ext[n].push_back(dT / (C_D[n] + dT * G_D[n] / 2.0) * ivv);
                                } else {
                                    i_int[n].push_back(1);
                                    i_ext[n].push_back(0);
                                }
                                if (C_L[n] > 0)
                                    v_lor[n].push_back(dT / C_L[n] / viv);
                                else
                                    v_lor[n].push_back(0);
                                if (L_L[n] > 0)
                                    i_lor[n].push_back(dT / L_L[n] / B.iv[B.at(n, pos)]);
                                else
                                    i_lor[n].push_back(0);
                            }
                        }
                    }
            A.count = (uint32_t)A.pos[0].size();
            auto pack = [&](std::vector<double>* src, std::vector<float>& dst, bool on) {
                dst.clear();
                if (!on) return;
                dst.resize(3 * (size_t)A.count);
                for (int n = 0; n < 3; ++n)
                    for (uint32_t i = 0; i < A.count; ++i) dst[(size_t)n * A.count + i] = (float)src[n][i];
            };
            pack(v_int, A.v_int, A.volt_on);
            pack(v_ext, A.v_ext, A.volt_on);
            pack(i_int, A.i_int, A.curr_on);
            pack(i_ext, A.i_ext, A.curr_on);
            pack(v_lor, A.v_lor, A.volt_lor_on);
            pack(i_lor, A.i_lor, A.curr_lor_on);
            op.ade.push_back(std::move(A));
        }
    }

    // ---- extension 9: lumped RLC elements (added last, openems.cpp:1095-1096);
    // fMax = GetCenterFreq() + GetCutOffFreq() (operator_ext_lumpedRLC.cpp:116-118):
    // f0 + fc of the Gaussian, f0 of the sinusoid.  The reference leaves
    // m_f0 / m_fc unset for the Dirac and step signals (and m_fc for the
    // sinusoid); they count as 0 here
    B.calc_rlc(S.f0 + S.fc, op.rlc);

    // ---- excitation signal: Excitation::buildExcitationSignal
    // (excitation.cpp:96-134) and CalcNyquistNum (tools/useful.cpp:30-36)
    op.signal_period_ts = 0;
    auto nyquist_num = [&](double fmax) -> uint32_t {
        if (fmax == 0) return UINT32_MAX;
        return (uint32_t)std::floor(1 / fmax / 2 / dT);
    };
    if (S.have_excite && S.excite_type == 0) {
        // CalcGaussianPulsExcitation (excitation.cpp:151-177)
        double f0 = S.f0, fc = S.fc;
        uint32_t Length = (uint32_t)std::ceil(2.0 * 9.0 / (2.0 * kPi * fc) / dT);
        if (S.nr_ts > 0 && Length > S.nr_ts) Length = S.nr_ts;
        op.sig_volt.resize(Length);
        op.sig_curr.resize(Length);
        for (uint32_t n = 0; n < Length; ++n) {
            double t = n * dT;
            op.sig_volt[n] = (float)(std::cos(2.0 * kPi * f0 * (t - 9.0 / (2.0 * kPi * fc))) *
                                     std::exp(-1 * std::pow(2.0 * kPi * fc * t / 3.0 - 3, 2)));
            t += 0.5 * dT;
            op.sig_curr[n] = (float)(std::cos(2.0 * kPi * f0 * (t - 9.0 / (2.0 * kPi * fc))) *
                                     std::exp(-1 * std::pow(2.0 * kPi * fc * t / 3.0 - 3, 2)));
        }
        op.nyquist = nyquist_num(f0 + fc);
    } else if (S.have_excite && S.excite_type == 1) {
        // CalcSinusExcitation (excitation.cpp:273-295): two periods
        const double f0 = S.f0;
        const uint32_t Length = (uint32_t)std::round(2.0 / f0 / dT);
        op.sig_volt.assign(Length, 0.f);
        op.sig_curr.assign(Length, 0.f);
        for (uint32_t n = 1; n < Length; ++n) {
            double t = n * dT;
            op.sig_volt[n] = (float)std::sin(2.0 * kPi * f0 * t);
            t += 0.5 * dT;
            op.sig_curr[n] = (float)std::sin(2.0 * kPi * f0 * t);
        }
        op.nyquist = nyquist_num(f0);
        // the engine's period p = int(GetSignalPeriod() / dT)
        // (engine_ext_excitation.cpp:45-46)
        op.signal_period_ts = (uint32_t)(int)((1 / f0) / dT);
    } else if (S.have_excite && S.excite_type == 10) {
        // CalcCustomExcitation (excitation.cpp:233-271): nr_ts samples of the
        // function at t = n dT (currents at t + dT / 2), Nyquist number of f0
        SignalExpr ex;
        std::string err;
        if (!ex.compile(S.exc_function, err)) {
            set_error("custom excitation: " + err);
            return FDTD_ERR_ARG;
        }
        op.sig_volt.resize(S.nr_ts);
        op.sig_curr.resize(S.nr_ts);
        for (uint32_t n = 0; n < S.nr_ts; ++n) {
            double t = n * dT;
            op.sig_volt[n] = (float)ex.eval(t);
            t += 0.5 * dT;
            op.sig_curr[n] = (float)ex.eval(t);
        }
        op.nyquist = nyquist_num(S.f0);
    } else if (S.have_excite) {
        // CalcDiracPulsExcitation / CalcStepExcitation (excitation.cpp:179-218)
        const float first = S.excite_type == 3 ? 1.f : 0.f;
        op.sig_volt = {first, 1.f};
        op.sig_curr = {first, 1.f};
        op.nyquist = 1;
    } else {
        op.sig_volt.clear();
        op.sig_curr.clear();
        op.nyquist = 1;
    }
    op.signal_length = (uint32_t)op.sig_volt.size();
    {
        // GetMaxExcitationTimestep (excitation.cpp:136-149)
        float maxAmp = 0;
        uint32_t maxStep = 0;
        for (uint32_t n = 0; n < op.signal_length; ++n)
            if (std::fabs(op.sig_volt[n]) > maxAmp) {
                maxAmp = std::fabs(op.sig_volt[n]);
                maxStep = n;
            }
        op.max_excite_ts = maxStep;
    }
    op.probe_interval = std::max<uint32_t>(1, op.nyquist / std::max<uint32_t>(1, S.oversampling));

    // ---- Mur ABC faces (Operator_Ext_Mur_ABC::SetDirection / BuildExtension,
    // operator_ext_mur_abc.cpp:88-195), in face order; the start timestep of
    // a face with an excitation on it follows Engine_Ext_Mur_ABC's
    // constructor (engine_ext_mur_abc.cpp:40-60)
    for (int f = 0; f < 6; ++f) {
        if (S.bc[f] != FDTD_BC_MUR) continue;
        MurFace M;
        M.ny = f / 2;
        M.top = f % 2;
        const int ny = M.ny, nP = (ny + 1) % 3, nPP = (ny + 2) % 3;
        if (N[ny] < 2) continue;
        M.line = M.top ? N[ny] - 1 : 0;
        M.shift = M.top ? N[ny] - 2 : 1;
        M.n[0] = N[nP];
        M.n[1] = N[nPP];
        M.cp.assign((size_t)M.n[0] * M.n[1], 0.f);
        M.cpp.assign((size_t)M.n[0] * M.n[1], 0.f);
        uint32_t pos[3] = {0, 0, 0};
        pos[ny] = M.line;
        const double delta = std::fabs(g.edge_length(ny, pos, false));
        int kind[3];
        kind[ny] = M.top ? SK_MURHI : SK_MURLO;
        kind[nP] = SK_LINE;
        kind[nPP] = SK_LINE;
        const double vph = S.mur_vph[f];
        for (pos[nP] = 0; pos[nP] < N[nP]; ++pos[nP])
            for (pos[nPP] = 0; pos[nPP] < N[nPP]; ++pos[nPP]) {
                const size_t k = (size_t)pos[nP] * M.n[1] + pos[nPP];
                const int w = B.mat_idx.lookup(kind, pos);
                double c0t;
                if (w >= 0) {
                    const Prim& p = S.prims[w];
                    c0t = vph > 0.0 ? vph * dT : kC0 * dT / std::sqrt(p.eps * p.mue);
                } else {
                    c0t = vph > 0.0 ? vph * dT : kC0 / std::sqrt(S.bg_eps * S.bg_mue) * dT;
                }
                M.cp[k] = (float)((c0t - delta) / (c0t + delta));
                M.cpp[k] = M.cp[k];
            }
        int maxDelay = -1;
        for (size_t n = 0; n < op.volt_exc.amp.size(); ++n)
            if ((op.volt_exc.dir[n] == nP || op.volt_exc.dir[n] == nPP) && op.volt_exc.index[ny][n] == M.line)
                maxDelay = std::max(maxDelay, (int)op.volt_exc.delay[n]);
        M.start_ts = maxDelay >= 0 ? (uint32_t)maxDelay + op.signal_length + 10 : 0;
        op.mur.push_back(std::move(M));
    }

    // ---- probes (openems.cpp:480-560 SetupProcessing)
    for (const Prim& p : S.prims) {
        if (p.kind != PK_PROBE) continue;
        fdtd_probe_desc d;
        std::memset(&d, 0, sizeof(d));
        d.type = p.probe_type;
        d.weight = p.weight;
        d.norm_dir = p.norm_dir;
        d.enabled = 1;
        bool si[3] = {false, false, false}, so[3] = {false, false, false};
        if (p.probe_type == 2 || p.probe_type == 3) {
            // ProcessFieldProbe: Processing::DefineStartStopCoord snaps the
            // box (SnapBox2Mesh with snap method 0, operator.cpp:289-314: the
            // corners sorted per axis) to the main mesh (E) or the dual mesh
            // (H, SetDualMesh, openems.cpp:520-524) and turns the probe off
            // when the box misses the grid; the probe reads the field at the
            // snapped lower corner (processfieldprobe.cpp:79-92)
            d.enabled = g.snap_box(p.start, p.stop, d.start, d.stop, p.probe_type == 3, 0, si, so) >= 0 ? 1 : 0;
        } else if (p.probe_type == 0) {
            // a voltage probe needs a box of dimension 1 (a line); any other
            // box is skipped with an error message (openems.cpp:481-486)
            int dimension = 0;
            for (int n = 0; n < 3; ++n) dimension += p.start[n] != p.stop[n];
            if (dimension != 1) continue;
            // ProcessVoltage::DefineStartStopCoord: SnapToMesh on the main mesh
            g.snap_mesh(p.start, d.start, false, si);
            g.snap_mesh(p.stop, d.stop, false, so);
        } else {
            // ProcessCurrent (dual mesh, snap method 1)
            int dim = g.snap_box(p.start, p.stop, d.start, d.stop, true, 1, si, so);
            if (dim < 0) d.enabled = 0;
            int nd = p.norm_dir;
            if (d.enabled) {
                if (nd < 0 || nd > 2) {
                    if (dim != 2)
                        d.enabled = 0;
                    else
                        for (int n = 0; n < 3; ++n)
                            if (d.stop[n] == d.start[n]) nd = n;
                } else {
                    for (int n = 0; n < 3; ++n) {
                        if (n == nd) continue;
                        if (p.start[n] == p.stop[n]) {
                            if ((g.line(n, d.start[n], true) > p.start[n]) && (d.start[n] > 0)) --d.start[n];
                            if ((g.line(n, d.start[n], true) < p.start[n]) && (d.stop[n] < N[n] - 1)) ++d.stop[n];
                        }
                    }
                }
                if (d.enabled && (nd < 0 || nd > 2 || d.start[nd] != d.stop[nd])) d.enabled = 0;
                d.norm_dir = nd;
            }
        }
        for (int n = 0; n < 3; ++n) {
            d.start_inside[n] = si[n];
            d.stop_inside[n] = so[n];
        }
        op.probes.push_back(d);
    }

    for (int n = 0; n < 3; ++n) {
        op.N[n] = N[n];
        op.lines[n] = S.lines[n];
    }
    op.unit = S.unit;
    op.dT = dT;
    op.vv.swap(B.vv);
    op.vi.swap(B.vi);
    op.ii.swap(B.ii);
    op.iv.swap(B.iv);
    return FDTD_OK;
}

}  // namespace wipems

using namespace wipems;

// ===================================================================== C ABI

extern "C" {

size_t fdtd_last_error(char* buf, size_t cap) {
    const std::string& e = last_error();
    if (buf && cap) {
        size_t n = std::min(cap - 1, e.size());
        std::memcpy(buf, e.data(), n);
        buf[n] = 0;
    }
    return e.size();
}

static bool check_box(const double* a, const double* b) { return a && b; }

int fdtd_scene_create(const double* lx, uint32_t nx, const double* ly, uint32_t ny, const double* lz,
                      uint32_t nz, double unit, fdtd_scene_t* out) {
    if (!out || !lx || !ly || !lz || nx < 2 || ny < 2 || nz < 2 || !(unit > 0)) {
        set_error("fdtd_scene_create: need >= 2 lines per axis and unit > 0");
        return FDTD_ERR_ARG;
    }
    const double* src[3] = {lx, ly, lz};
    uint32_t cnt[3] = {nx, ny, nz};
    for (int a = 0; a < 3; ++a)
        for (uint32_t i = 1; i < cnt[a]; ++i)
            if (!(src[a][i] > src[a][i - 1])) {
                set_error("fdtd_scene_create: mesh lines must be strictly increasing");
                return FDTD_ERR_ARG;
            }
    fdtd_scene_s* s = new (std::nothrow) fdtd_scene_s();
    if (!s) return FDTD_ERR_NOMEM;
    for (int a = 0; a < 3; ++a) s->lines[a].assign(src[a], src[a] + cnt[a]);
    s->unit = unit;
    *out = s;
    return FDTD_OK;
}

int fdtd_scene_destroy(fdtd_scene_t s) {
    delete s;
    return FDTD_OK;
}

int fdtd_scene_set_background(fdtd_scene_t s, double eps_r, double mue_r, double kappa, double sigma) {
    if (!s) return FDTD_ERR_ARG;
    s->bg_eps = eps_r;
    s->bg_mue = mue_r;
    s->bg_kappa = kappa;
    s->bg_sigma = sigma;
    return FDTD_OK;
}

int fdtd_scene_set_boundary(fdtd_scene_t s, const int bc[6], const uint32_t pml_size[6]) {
    if (!s || !bc) return FDTD_ERR_ARG;
    for (int i = 0; i < 6; ++i) {
        if (bc[i] < -1 || bc[i] > 3) {
            set_error("fdtd_scene_set_boundary: unknown boundary code");
            return FDTD_ERR_ARG;
        }
        s->bc[i] = bc[i];
        // openEMS gives every face a PML size of 8 (openems.cpp:101) and
        // changes it only for PML_n faces; its UPML build reads the size of a
        // face that is not PML too (the grading of the opposite face,
        // operator_ext_upml.cpp:337, and the y/z slab ranges, :163)
        s->pml_size[i] = (bc[i] == FDTD_BC_PML && pml_size) ? pml_size[i] : 8;
    }
    return FDTD_OK;
}

int fdtd_scene_num_dumps(fdtd_scene_t s, uint32_t* n) {
    if (!s || !n) return FDTD_ERR_ARG;
    *n = (uint32_t)s->dumps.size();
    return FDTD_OK;
}

int fdtd_scene_get_dump(fdtd_scene_t s, uint32_t k, fdtd_scene_dump* out) {
    if (!s || !out || k >= s->dumps.size()) {
        set_error("fdtd_scene_get_dump: no such dump");
        return FDTD_ERR_ARG;
    }
    const DumpSpec& d = s->dumps[k];
    std::memset(out, 0, sizeof(*out));
    std::strncpy(out->name, d.name.c_str(), sizeof(out->name) - 1);
    out->field = d.field;
    out->interp = d.interp;
    out->file_type = d.file_type;
    for (int a = 0; a < 3; ++a) {
        out->start[a] = d.start[a];
        out->stop[a] = d.stop[a];
        out->step[a] = d.step[a];
    }
    return FDTD_OK;
}

int fdtd_scene_set_mur_velocity(fdtd_scene_t s, const double v_phase[6]) {
    if (!s || !v_phase) return FDTD_ERR_ARG;
    for (int i = 0; i < 6; ++i) {
        if (!(v_phase[i] >= 0)) {
            set_error("fdtd_scene_set_mur_velocity: phase velocities must be >= 0");
            return FDTD_ERR_ARG;
        }
        s->mur_vph[i] = v_phase[i];
    }
    return FDTD_OK;
}

int fdtd_scene_set_gauss_excite(fdtd_scene_t s, double f0, double fc, uint32_t nr_ts) {
    if (!s || !(fc > 0) || f0 < 0) {
        set_error("fdtd_scene_set_gauss_excite: need fc > 0, f0 >= 0");
        return FDTD_ERR_ARG;
    }
    s->f0 = f0;
    s->fc = fc;
    s->nr_ts = nr_ts;
    s->excite_type = 0;
    s->have_excite = true;
    return FDTD_OK;
}

int fdtd_scene_set_sinus_excite(fdtd_scene_t s, double f0, uint32_t nr_ts) {
    if (!s || !(f0 > 0) || nr_ts == 0) {
        set_error("fdtd_scene_set_sinus_excite: need f0 > 0 and nr_ts > 0");
        return FDTD_ERR_ARG;
    }
    s->f0 = f0;
    s->fc = 0;
    s->nr_ts = nr_ts;
    s->excite_type = 1;
    s->have_excite = true;
    return FDTD_OK;
}

static int set_unit_excite(fdtd_scene_t s, int type, double f_max, uint32_t nr_ts, const char* name) {
    if (!s || f_max < 0) {
        set_error(std::string(name) + ": need f_max >= 0");
        return FDTD_ERR_ARG;
    }
    s->f0 = 0;
    s->fc = 0;
    s->f_max = f_max;
    s->nr_ts = nr_ts;
    s->excite_type = type;
    s->have_excite = true;
    return FDTD_OK;
}

int fdtd_scene_set_custom_excite(fdtd_scene_t s, const char* function, double f0, double f_max, uint32_t nr_ts) {
    if (!s || !function || nr_ts == 0 || !(f0 >= 0)) {
        set_error("fdtd_scene_set_custom_excite: need a function, f0 >= 0 and nr_ts > 0");
        return FDTD_ERR_ARG;
    }
    SignalExpr ex;
    std::string err;
    if (!ex.compile(function, err)) {
        set_error("fdtd_scene_set_custom_excite: " + err);
        return FDTD_ERR_ARG;
    }
    s->f0 = f0;
    s->fc = 0;
    s->f_max = f_max;
    s->nr_ts = nr_ts;
    s->exc_function = function;
    s->excite_type = 10;
    s->have_excite = true;
    return FDTD_OK;
}

int fdtd_scene_set_dirac_excite(fdtd_scene_t s, double f_max, uint32_t nr_ts) {
    return set_unit_excite(s, 2, f_max, nr_ts, "fdtd_scene_set_dirac_excite");
}

int fdtd_scene_set_step_excite(fdtd_scene_t s, double f_max, uint32_t nr_ts) {
    return set_unit_excite(s, 3, f_max, nr_ts, "fdtd_scene_set_step_excite");
}

int fdtd_scene_set_oversampling(fdtd_scene_t s, uint32_t os) {
    if (!s || os == 0) return FDTD_ERR_ARG;
    s->oversampling = os;
    return FDTD_OK;
}

static Prim make_box(int kind, int prio, const double* a, const double* b) {
    Prim p;
    p.kind = kind;
    p.priority = prio;
    for (int n = 0; n < 3; ++n) {
        p.start[n] = a[n];
        p.stop[n] = b[n];
        p.bmin[n] = std::fmin(a[n], b[n]);
        p.bmax[n] = std::fmax(a[n], b[n]);
    }
    return p;
}

int fdtd_scene_add_material(fdtd_scene_t s, int prio, const double start[3], const double stop[3],
                            double eps_r, double kappa, double mue_r, double sigma) {
    if (!s || !check_box(start, stop) || !(eps_r > 0) || !(mue_r > 0) || kappa < 0 || sigma < 0) {
        set_error("fdtd_scene_add_material: invalid box or material");
        return FDTD_ERR_ARG;
    }
    Prim p = make_box(PK_MATERIAL, prio, start, stop);
    p.eps = eps_r;
    p.kappa = kappa;
    p.mue = mue_r;
    p.sigma = sigma;
    s->prims.push_back(p);
    return FDTD_OK;
}

int fdtd_scene_add_metal(fdtd_scene_t s, int prio, const double start[3], const double stop[3]) {
    if (!s || !check_box(start, stop)) return FDTD_ERR_ARG;
    s->prims.push_back(make_box(PK_METAL, prio, start, stop));
    return FDTD_OK;
}

int fdtd_scene_add_lumped(fdtd_scene_t s, int prio, const double start[3], const double stop[3], int dir,
                          double R, double C, int caps) {
    if (!s || !check_box(start, stop) || dir < 0 || dir > 2) {
        set_error("fdtd_scene_add_lumped: invalid box or direction");
        return FDTD_ERR_ARG;
    }
    Prim p = make_box(PK_LUMPED, prio, start, stop);
    p.ny = dir;
    p.R = R;
    p.C = C;
    p.caps = caps != 0;
    s->prims.push_back(p);
    return FDTD_OK;
}

int fdtd_scene_add_lumped_rlc(fdtd_scene_t s, int prio, const double start[3], const double stop[3], int dir,
                              int type, double R, double L, double C, int caps) {
    if (!s || !check_box(start, stop) || dir < 0 || dir > 2 || type < FDTD_LE_INVALID || type > FDTD_LE_SERIES) {
        set_error("fdtd_scene_add_lumped_rlc: invalid box, direction or type");
        return FDTD_ERR_ARG;
    }
    Prim p = make_box(PK_LUMPED, prio, start, stop);
    p.ny = dir;
    p.le_type = type;
    p.R = R;
    p.L = L;
    p.C = C;
    p.caps = caps != 0;
    s->prims.push_back(p);
    return FDTD_OK;
}

int fdtd_scene_add_excitation(fdtd_scene_t s, int prio, const double start[3], const double stop[3],
                              int exc_type, const double vec[3], double delay) {
    if (!s || !check_box(start, stop) || !vec || exc_type < 0 || exc_type > 3 || delay < 0) {
        set_error("fdtd_scene_add_excitation: invalid arguments");
        return FDTD_ERR_ARG;
    }
    Prim p = make_box(PK_EXCITATION, prio, start, stop);
    p.exc_type = exc_type;
    for (int n = 0; n < 3; ++n) p.exc_vec[n] = vec[n];
    p.delay = delay;
    s->prims.push_back(p);
    return FDTD_OK;
}

int fdtd_scene_add_lorentz_material(fdtd_scene_t s, int prio, const double start[3], const double stop[3],
                                    double eps_r, double kappa, double mue_r, double sigma, int order,
                                    const double* eps_plasma_f, const double* eps_relax_t,
                                    const double* eps_lor_pole_f, const double* mue_plasma_f,
                                    const double* mue_relax_t, const double* mue_lor_pole_f) {
    if (!s || !check_box(start, stop) || order < 1 || order > kMaxDispOrder || !(eps_r > 0) || !(mue_r > 0)) {
        set_error("fdtd_scene_add_lorentz_material: invalid arguments (order 1..4)");
        return FDTD_ERR_ARG;
    }
    Prim p = make_box(PK_MATERIAL, prio, start, stop);
    p.eps = eps_r;
    p.kappa = kappa;
    p.mue = mue_r;
    p.sigma = sigma;
    p.lorentz = true;
    p.disp_order = order;
    for (int o = 0; o < order; ++o) {
        p.eps_plasma_f[o] = eps_plasma_f ? eps_plasma_f[o] : 0;
        p.eps_relax_t[o] = eps_relax_t ? eps_relax_t[o] : 0;
        p.eps_lor_pole_f[o] = eps_lor_pole_f ? eps_lor_pole_f[o] : 0;
        p.mue_plasma_f[o] = mue_plasma_f ? mue_plasma_f[o] : 0;
        p.mue_relax_t[o] = mue_relax_t ? mue_relax_t[o] : 0;
        p.mue_lor_pole_f[o] = mue_lor_pole_f ? mue_lor_pole_f[o] : 0;
    }
    s->prims.push_back(p);
    return FDTD_OK;
}

int fdtd_scene_add_lorentz(fdtd_scene_t s, int prio, const double start[3], const double stop[3], double eps_r,
                           double kappa, double mue_r, double sigma, int order, const double* plasma_f,
                           const double* relax_t, const double* pole_f) {
    if (!plasma_f) {
        set_error("fdtd_scene_add_lorentz: invalid arguments (order 1..4)");
        return FDTD_ERR_ARG;
    }
    return fdtd_scene_add_lorentz_material(s, prio, start, stop, eps_r, kappa, mue_r, sigma, order, plasma_f,
                                           relax_t, pole_f, nullptr, nullptr, nullptr);
}

int fdtd_scene_add_probe(fdtd_scene_t s, int type, const double start[3], const double stop[3], double weight,
                         int norm_dir) {
    if (!s || !check_box(start, stop) || type < 0 || type > 3 || norm_dir < -1 || norm_dir > 2) {
        set_error("fdtd_scene_add_probe: type must be 0 (voltage), 1 (current), 2 (E field) or 3 (H field)");
        return FDTD_ERR_ARG;
    }
    Prim p = make_box(PK_PROBE, 0, start, stop);
    p.probe_type = type;
    p.weight = weight;
    p.norm_dir = norm_dir;
    s->prims.push_back(p);
    return FDTD_OK;
}

int fdtd_operator_build(fdtd_scene_t scene, int num_threads, fdtd_operator_t* out) {
    if (!scene || !out) return FDTD_ERR_ARG;
    if (num_threads <= 0) num_threads = (int)std::max(1u, std::thread::hardware_concurrency());
    fdtd_operator_s* op = new (std::nothrow) fdtd_operator_s();
    if (!op) return FDTD_ERR_NOMEM;
    int rc;
    try {
        rc = build_operator(*scene, num_threads, *op);
    } catch (const std::bad_alloc&) {
        set_error("fdtd_operator_build: host allocation failed");
        rc = FDTD_ERR_NOMEM;
    }
    if (rc != FDTD_OK) {
        delete op;
        return rc;
    }
    *out = op;
    return FDTD_OK;
}

int fdtd_operator_destroy(fdtd_operator_t op) {
    delete op;
    return FDTD_OK;
}

int fdtd_operator_get_info(fdtd_operator_t op, fdtd_operator_info* info) {
    if (!op || !info) return FDTD_ERR_ARG;
    std::memset(info, 0, sizeof(*info));
    for (int n = 0; n < 3; ++n) info->num_lines[n] = op->N[n];
    info->dT = op->dT;
    info->unit = op->unit;
    info->nyquist = op->nyquist;
    info->probe_interval = op->probe_interval;
    info->signal_length = op->signal_length;
    info->max_excite_ts = op->max_excite_ts;
    info->num_upml = (uint32_t)op->upml.size();
    info->ade_order = (uint32_t)op->ade.size();
    info->volt_exc_count = (uint32_t)op->volt_exc.amp.size();
    info->curr_exc_count = (uint32_t)op->curr_exc.amp.size();
    info->num_probes = (uint32_t)op->probes.size();
    info->num_cells = (double)op->N[0] * op->N[1] * op->N[2];
    return FDTD_OK;
}

int fdtd_operator_describe(fdtd_operator_t op, fdtd_op_desc* d) {
    if (!op || !d) return FDTD_ERR_ARG;
    std::memset(d, 0, sizeof(*d));
    for (int n = 0; n < 3; ++n) d->num_lines[n] = op->N[n];
    d->dT = op->dT;
    d->vv = op->vv.data();
    d->vi = op->vi.data();
    d->ii = op->ii.data();
    d->iv = op->iv.data();
    op->upml_desc.resize(op->upml.size());
    for (size_t k = 0; k < op->upml.size(); ++k) {
        fdtd_upml_desc& u = op->upml_desc[k];
        const UpmlSlab& s = op->upml[k];
        for (int n = 0; n < 3; ++n) {
            u.start[n] = s.start[n];
            u.num_lines[n] = s.num_lines[n];
        }
        u.vv = s.vv.data(); u.vvfo = s.vvfo.data(); u.vvfn = s.vvfn.data();
        u.ii = s.ii.data(); u.iifo = s.iifo.data(); u.iifn = s.iifn.data();
    }
    d->num_upml = (uint32_t)op->upml.size();
    d->upml = op->upml_desc.empty() ? nullptr : op->upml_desc.data();
    op->ade_desc.resize(op->ade.size());
    for (size_t k = 0; k < op->ade.size(); ++k) {
        fdtd_ade_desc& a = op->ade_desc[k];
        const AdeOrder& s = op->ade[k];
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
    d->volt_count = (uint32_t)op->volt_exc.amp.size();
    d->curr_count = (uint32_t)op->curr_exc.amp.size();
    for (int n = 0; n < 3; ++n) {
        d->volt_index[n] = op->volt_exc.index[n].data();
        d->curr_index[n] = op->curr_exc.index[n].data();
    }
    d->volt_dir = op->volt_exc.dir.data();
    d->volt_amp = op->volt_exc.amp.data();
    d->volt_delay = op->volt_exc.delay.data();
    d->curr_dir = op->curr_exc.dir.data();
    d->curr_amp = op->curr_exc.amp.data();
    d->curr_delay = op->curr_exc.delay.data();
    op->mur_desc.resize(op->mur.size());
    for (size_t k = 0; k < op->mur.size(); ++k) {
        const MurFace& M = op->mur[k];
        fdtd_mur_desc& m = op->mur_desc[k];
        m.ny = M.ny;
        m.top = M.top;
        m.line = M.line;
        m.shift = M.shift;
        m.n_p = M.n[0];
        m.n_pp = M.n[1];
        m.coef_p = M.cp.data();
        m.coef_pp = M.cpp.data();
        m.start_ts = M.start_ts;
    }
    d->num_mur = (uint32_t)op->mur.size();
    d->mur = op->mur_desc.empty() ? nullptr : op->mur_desc.data();
    {
        const RlcList& r = op->rlc;
        fdtd_rlc_desc& q = op->rlc_desc;
        q.count = (uint32_t)r.size();
        for (int n = 0; n < 3; ++n) q.pos[n] = r.pos[n].data();
        q.dir = r.dir.data();
        q.ilv = r.ilv.data(); q.i2v = r.i2v.data();
        q.vv2 = r.vv2.data(); q.vj1 = r.vj1.data(); q.vj2 = r.vj2.data(); q.vvd = r.vvd.data();
        q.ib0 = r.ib0.data(); q.b1 = r.b1.data(); q.b2 = r.b2.data();
        d->rlc = q.count ? &op->rlc_desc : nullptr;
    }
    d->signal_length = op->signal_length;
    d->signal_volt = op->sig_volt.data();
    d->signal_curr = op->sig_curr.data();
    d->signal_period_ts = op->signal_period_ts;
    for (int n = 0; n < 3; ++n) d->lines[n] = op->lines[n].data();
    d->unit = op->unit;
    return FDTD_OK;
}

int fdtd_operator_get_probe(fdtd_operator_t op, uint32_t i, fdtd_probe_desc* out) {
    if (!op || !out || i >= op->probes.size()) return FDTD_ERR_ARG;
    *out = op->probes[i];
    return FDTD_OK;
}

}  // extern "C"
