// Host-side compression of a reference-form operator into per-node E/H
// tuple indices and coefficient tables (see cop.h).  Runs without a GPU; the
// index arrays go to pinned memory when a CUDA device is present so that the
// engine upload is a plain DMA.
#include <cuda_runtime_api.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "cop.h"
#include "fdtd_host.h"

fdtd_cop_s::~fdtd_cop_s() {
    for (wipems::HalfTables* h : {&E, &H}) {
        if (!h->idx) continue;
        if (h->pinned)
            cudaFreeHost(h->idx);
        else
            std::free(h->idx);
        h->idx = nullptr;
    }
}

namespace wipems {
namespace {

// tuples are hashed and compared over their first `bytes` bytes: the base
// 128 bytes, or the whole tuple when the operator has dispersion orders > 1
// (the rest is zero otherwise)
struct TupleHash {
    size_t bytes = kTupleBaseBytes;
    size_t operator()(const HalfTuple& t) const {
        const uint64_t* p = reinterpret_cast<const uint64_t*>(&t);
        uint64_t h = 1469598103934665603ull;
        for (size_t i = 0; i < bytes / 8; ++i) h ^= p[i] + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2);
        return (size_t)h;
    }
};
struct TupleEq {
    size_t bytes = kTupleBaseBytes;
    bool operator()(const HalfTuple& a, const HalfTuple& b) const { return std::memcmp(&a, &b, bytes) == 0; }
};
using TupleMap = std::unordered_map<HalfTuple, uint32_t, TupleHash, TupleEq>;

TupleMap make_map(size_t bytes) { return TupleMap(64, TupleHash{bytes}, TupleEq{bytes}); }

// Operator::GetEdgeLength (main / dual) from the mesh lines, operator.cpp:136-185
double edge_len(const double* l, uint32_t N, uint32_t pos, bool dual, double unit) {
    auto line = [&](uint32_t p, bool du) -> double {
        if (!du) return l[p];
        if (p < N - 1) return 0.5 * (l[p] + l[p + 1]);
        return l[p] + 0.5 * (l[p] - l[p - 1]);
    };
    double d;
    if (!dual)
        d = (pos < N - 1) ? line(pos + 1, false) - line(pos, false) : line(pos, false) - line(pos - 1, false);
    else
        d = (pos > 0) ? line(pos, true) - line(pos - 1, true) : line(1, false) - line(0, false);
    return d * unit;
}

bool mesh_uniform(const fdtd_op_desc* d) {
    for (int a = 0; a < 3; ++a) {
        const double* l = d->lines[a];
        const uint32_t N = d->num_lines[a];
        const double d0 = l[1] - l[0];
        for (uint32_t i = 1; i + 1 < N; ++i)
            if (std::fabs((l[i + 1] - l[i]) - d0) > 1e-9 * std::fabs(d0)) return false;
    }
    return true;
}

struct Plan {
    const fdtd_op_desc* d;
    uint32_t N[3];  // the operator's grid (reference axes)
    int rot = 0;    // device axis a holds reference axis (a + rot) % 3
    uint32_t D[3];  // the device grid: D[a] = N[(a + rot) % 3]
    size_t NN;
    bool geo;
    const float* gf[4][3];  // dE, iD, dH, iM per axis (float arrays in cop->geom)
    std::vector<int8_t> slab;
    std::vector<int32_t> ade;                 // order 0: node -> position in the order's list
    std::vector<int32_t> adex[kExtraOrders];  // orders 1..3
    size_t key_bytes = kTupleBaseBytes;
    std::unordered_map<uint64_t, uint32_t> vexc, cexc;
};

int prepare(const fdtd_op_desc* d, Plan& P) {
    const uint32_t Nx = P.N[0], Ny = P.N[1], Nz = P.N[2];
    if (d->num_upml) {
        if (d->num_upml > 127) {
            set_error("too many UPML slabs");
            return FDTD_ERR_ARG;
        }
        P.slab.assign(P.NN, -1);
        for (uint32_t s = 0; s < d->num_upml; ++s) {
            const fdtd_upml_desc& u = d->upml[s];
            for (int a = 0; a < 3; ++a)
                if (u.start[a] + u.num_lines[a] > P.N[a]) {
                    set_error("UPML slab exceeds the grid");
                    return FDTD_ERR_ARG;
                }
            for (uint32_t x = 0; x < u.num_lines[0]; ++x)
                for (uint32_t y = 0; y < u.num_lines[1]; ++y)
                    for (uint32_t z = 0; z < u.num_lines[2]; ++z) {
                        size_t gi = ((size_t)(x + u.start[0]) * Ny + (y + u.start[1])) * Nz + (z + u.start[2]);
                        if (P.slab[gi] >= 0) {
                            // openEMS builds such slabs when the x-max UPML is
                            // thicker than the x-min size (8 for a face that is
                            // not PML): the y and z slabs end size[0]+1 lines
                            // before the x-max face (operator_ext_upml.cpp:163),
                            // so they run into the x-max slab and both
                            // extensions update the nodes they share.  One UPML
                            // update per node is all the fused kernels do.
                            set_error("UPML slabs overlap (the x-max UPML is thicker than the x-min size -- 8 for a "
                                      "face that is not PML -- so the y/z slabs reach into it, as openEMS builds "
                                      "them); keep the x-max UPML no thicker than that");
                            return FDTD_ERR_ARG;
                        }
                        P.slab[gi] = (int8_t)s;
                    }
        }
    }
    if (d->num_ade_orders > (uint32_t)kMaxDispOrder) {
        set_error("dispersion order > 4 is not provided");
        return FDTD_ERR_UNSUPPORTED;
    }
    for (uint32_t o = 0; o < d->num_ade_orders; ++o) {
        const fdtd_ade_desc& A = d->ade[o];
        std::vector<int32_t>& m = o == 0 ? P.ade : P.adex[o - 1];
        if (!A.volt_on && !A.curr_on) continue;  // the order's hooks are off (engine_ext_lorentzmaterial.cpp:83,132)
        m.assign(P.NN, -1);
        for (uint32_t i = 0; i < A.count; ++i) {
            uint32_t x = A.pos[0][i], y = A.pos[1][i], z = A.pos[2][i];
            if (x >= Nx || y >= Ny || z >= Nz) {
                set_error("ADE position outside the grid");
                return FDTD_ERR_ARG;
            }
            m[((size_t)x * Ny + y) * Nz + z] = (int32_t)i;
        }
        if (o > 0) P.key_bytes = sizeof(HalfTuple);
    }
    for (int half = 0; half < 2; ++half) {
        const uint32_t cnt = half ? d->curr_count : d->volt_count;
        for (uint32_t i = 0; i < cnt; ++i) {
            const uint32_t x = (half ? d->curr_index : d->volt_index)[0][i];
            const uint32_t y = (half ? d->curr_index : d->volt_index)[1][i];
            const uint32_t z = (half ? d->curr_index : d->volt_index)[2][i];
            const uint16_t dir = (half ? d->curr_dir : d->volt_dir)[i];
            const uint32_t lim = half ? 1 : 0;
            if (x >= Nx - lim || y >= Ny - lim || z >= Nz - lim || dir > 2) {
                set_error(half ? "current excitation outside the current domain" : "voltage excitation outside the grid");
                return FDTD_ERR_ARG;
            }
            const uint64_t key = (((uint64_t)x * Ny + y) * Nz + z) * 3 + dir;
            auto& m = half ? P.cexc : P.vexc;
            if (m.count(key)) {
                set_error("duplicate excitation on one edge");
                return FDTD_ERR_ARG;
            }
            m[key] = i;
        }
    }
    return FDTD_OK;
}

// Builds the E (half = 0) or H (half = 1) tuple of a node.
// (x, y, z) and gi are the node in the reference's axes; slot k of every
// per-component group holds reference component (k + rot) % 3, the device
// component k.
void make_tuple(const Plan& P, int half, uint32_t x, uint32_t y, uint32_t z, size_t gi, HalfTuple& t) {
    const fdtd_op_desc* d = P.d;
    std::memset(&t, 0, P.key_bytes);
    const float* c1 = half ? d->ii : d->vv;
    const float* c2 = half ? d->iv : d->vi;
    const uint32_t pos[3] = {x, y, z};
    int src[3];  // reference component of device slot k
    for (int k = 0; k < 3; ++k) src[k] = (k + P.rot) % 3;
    for (int k = 0; k < 3; ++k) {
        const int n = src[k];
        t.c[k] = c1[n * P.NN + gi];
        float v = c2[n * P.NN + gi];
        if (P.geo && v != 0.f) {
            const int nP = (n + 1) % 3, nPP = (n + 2) % 3;
            const float* a0 = P.gf[half ? 2 : 0][n];
            const float* a1 = P.gf[half ? 3 : 1][nP];
            const float* a2 = P.gf[half ? 3 : 1][nPP];
            const double g = (double)a0[pos[n]] * (double)a1[pos[nP]] * (double)a2[pos[nPP]];
            v = (float)((double)v / g);
        }
        t.c[3 + k] = v;
        t.xd[k] = -1;
    }
    if (!P.slab.empty() && P.slab[gi] >= 0) {
        const fdtd_upml_desc& u = d->upml[P.slab[gi]];
        const size_t nloc = (size_t)u.num_lines[0] * u.num_lines[1] * u.num_lines[2];
        const size_t li =
            ((size_t)(x - u.start[0]) * u.num_lines[1] + (y - u.start[1])) * u.num_lines[2] + (z - u.start[2]);
        const float* a = half ? u.ii : u.vv;
        const float* b = half ? u.iifo : u.vvfo;
        const float* c = half ? u.iifn : u.vvfn;
        for (int k = 0; k < 3; ++k) {
            const int n = src[k];
            t.u[k] = a[n * nloc + li];
            t.u[3 + k] = b[n * nloc + li];
            t.u[6 + k] = c[n * nloc + li];
        }
        t.flags |= TF_UPML;
    }
    // ADE terms of each order whose list holds the node and whose hooks run
    // for this half (m_volt_ADE_On / m_curr_ADE_On of the order)
    for (uint32_t o = 0; o < d->num_ade_orders; ++o) {
        const std::vector<int32_t>& m = o == 0 ? P.ade : P.adex[o - 1];
        if (m.empty() || m[gi] < 0) continue;
        const fdtd_ade_desc& A = d->ade[o];
        const uint32_t i = (uint32_t)m[gi];
        const bool on = half ? A.curr_on : A.volt_on;
        if (!on) continue;
        const float* ai = half ? A.i_int : A.v_int;
        const float* ae = half ? A.i_ext : A.v_ext;
        const float* al = half ? A.i_lor : A.v_lor;
        const bool lor_on = half ? A.curr_lor_on : A.volt_lor_on;
        float* dst = o == 0 ? t.a : t.ax[o - 1];
        bool lor = false;
        for (int k = 0; k < 3; ++k) {
            const int n = src[k];
            dst[k] = ai[n * A.count + i];
            dst[3 + k] = ae[n * A.count + i];
            dst[6 + k] = (lor_on && al) ? al[n * A.count + i] : 0.f;
            if (dst[6 + k] != 0.f) lor = true;
        }
        if (o == 0)
            t.flags |= TF_ADE | (lor ? TF_LOR : 0u);
        else
            t.flags |= (TF_ADEX << (o - 1)) | (lor ? (TF_LORX << (o - 1)) : 0u);
    }
    const auto& m = half ? P.cexc : P.vexc;
    if (!m.empty())
        for (int k = 0; k < 3; ++k) {
            auto it = m.find((uint64_t)gi * 3 + src[k]);
            if (it != m.end()) {
                t.x[k] = (half ? d->curr_amp : d->volt_amp)[it->second];
                t.xd[k] = (int32_t)(half ? d->curr_delay : d->volt_delay)[it->second];
                t.flags |= TF_EXC;
            }
        }
}

// The cyclic relabelling of the axes that fits the grid best to the
// kernels' tiles (32 z-lanes by 4 rows): the EC update is the same under
// x -> y -> z -> x (every component's update has the same operation order
// relative to its own axis), so a rotated grid gives bit-identical fields.
// Cost = padded node count; a rotation is taken when it saves over 3 %.
int choose_rotation(const uint32_t N[3], int want) {
    if (want >= 0 && want <= 2) return want;
    auto cost = [&](int r) {
        const uint64_t dx = N[r % 3], dy = N[(1 + r) % 3], dz = N[(2 + r) % 3];
        return (double)dx * (double)((dy + 3) / 4 * 4) * (double)((dz + 31) / 32 * 32);
    };
    int best = 0;
    for (int r = 1; r < 3; ++r)
        if (cost(r) < cost(best)) best = r;
    return cost(best) < 0.97 * cost(0) ? best : 0;
}

// ---- factorized mode: snapping of rounding variants ------------------------
// On a graded mesh the factorized VI = vi / g, and the ADE and UPML terms,
// come out of the operator's float arithmetic with last-bit variants that
// differ from node to node (the geometric factors cancel in exact
// arithmetic, not in the rounded one).  Within each coefficient kind the
// variants are mapped onto the most frequent value at most kSnapUlps float
// steps away, so tuples that differ only by such variants merge (D192: about
// 300 K voltage tuples -> a table that fits the uint16 index).  Zero and
// non-finite values are never moved; the map depends on the operator alone
// (node counts, values), not on threads or order.
constexpr int64_t kSnapUlps = 1;

inline int64_t float_order(float f) {  // adjacent floats differ by 1
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return (u >> 31) ? -(int64_t)(u & 0x7fffffffu) : (int64_t)u;
}

// the coefficient kind of every snapped slot of a tuple: VI|IV, the three
// ADE kinds and the three UPML kinds (vv|ii stay exact)
constexpr int kSnapKinds = 7;
template <class F>
void for_snap_slots(HalfTuple& t, F&& f) {
    for (int n = 0; n < 3; ++n) f(0, t.c[3 + n]);
    if (t.flags & TF_ADE)
        for (int k = 0; k < 9; ++k) f(1 + k / 3, t.a[k]);
    for (int o = 0; o < kExtraOrders; ++o)
        if (t.flags & (TF_ADEX << o))
            for (int k = 0; k < 9; ++k) f(1 + k / 3, t.ax[o][k]);
    if (t.flags & TF_UPML)
        for (int k = 0; k < 9; ++k) f(4 + k / 3, t.u[k]);
}

// Snaps the tuples (weighted by the nodes using them), merges the tuples
// that became equal; returns old tuple id -> new tuple id.
std::vector<uint32_t> snap_tuples(std::vector<HalfTuple>& tuples, const std::vector<uint64_t>& uses,
                                  size_t key_bytes) {
    std::unordered_map<uint32_t, uint64_t> hist[kSnapKinds];
    for (size_t k = 0; k < tuples.size(); ++k) {
        HalfTuple t = tuples[k];
        for_snap_slots(t, [&](int kind, float& v) {
            if (v == 0.f || !std::isfinite(v)) return;
            uint32_t b;
            std::memcpy(&b, &v, 4);
            hist[kind][b] += uses[k];
        });
    }
    std::unordered_map<uint32_t, uint32_t> to[kSnapKinds];
    for (int kind = 0; kind < kSnapKinds; ++kind) {
        struct V {
            int64_t ord;
            uint32_t bits;
            uint64_t cnt;
        };
        std::vector<V> vals;
        vals.reserve(hist[kind].size());
        for (const auto& kv : hist[kind]) {
            float f;
            std::memcpy(&f, &kv.first, 4);
            vals.push_back(V{float_order(f), kv.first, kv.second});
        }
        std::sort(vals.begin(), vals.end(), [](const V& a, const V& b) { return a.ord < b.ord; });
        std::vector<size_t> order(vals.size());
        for (size_t i = 0; i < order.size(); ++i) order[i] = i;
        std::sort(order.begin(), order.end(), [&](size_t a, size_t b) {
            return vals[a].cnt != vals[b].cnt ? vals[a].cnt > vals[b].cnt : vals[a].ord < vals[b].ord;
        });
        std::vector<int64_t> rep(vals.size(), -1);
        for (size_t i : order) {
            if (rep[i] >= 0) continue;
            rep[i] = (int64_t)i;
            for (size_t j = i; j-- > 0 && vals[i].ord - vals[j].ord <= kSnapUlps;)
                if (rep[j] < 0) rep[j] = (int64_t)i;
            for (size_t j = i + 1; j < vals.size() && vals[j].ord - vals[i].ord <= kSnapUlps; ++j)
                if (rep[j] < 0) rep[j] = (int64_t)i;
        }
        for (size_t i = 0; i < vals.size(); ++i) to[kind][vals[i].bits] = vals[(size_t)rep[i]].bits;
    }
    TupleMap merged = make_map(key_bytes);
    std::vector<HalfTuple> out;
    std::vector<uint32_t> newid(tuples.size());
    for (size_t k = 0; k < tuples.size(); ++k) {
        HalfTuple t = tuples[k];
        for_snap_slots(t, [&](int kind, float& v) {
            if (v == 0.f || !std::isfinite(v)) return;
            uint32_t b;
            std::memcpy(&b, &v, 4);
            const uint32_t r = to[kind].at(b);
            std::memcpy(&v, &r, 4);
        });
        auto it = merged.find(t);
        if (it == merged.end()) {
            newid[k] = (uint32_t)out.size();
            merged.emplace(t, newid[k]);
            out.push_back(t);
        } else {
            newid[k] = it->second;
        }
    }
    tuples.swap(out);
    return newid;
}

void pack(const std::vector<HalfTuple>& tuples, HalfTables& T) {
    const size_t n = tuples.size();
    T.num_tuples = (uint32_t)n;
    T.main.assign(n * TAB_MAIN * 4, 0.f);
    T.exc.assign(n * TAB_EXC * 4, 0.f);
    for (const HalfTuple& t : tuples) {
        T.any_upml |= (t.flags & TF_UPML) != 0;
        T.any_ade |= (t.flags & TF_ADE) != 0;
        T.any_lor |= (t.flags & TF_LOR) != 0;
        T.any_exc |= (t.flags & TF_EXC) != 0;
        for (int o = 0; o < kExtraOrders; ++o)
            if (t.flags & (TF_ADEX << o)) T.adex_orders = std::max(T.adex_orders, o + 1);
        T.any_lorx |= (t.flags & (7u * TF_LORX)) != 0;
    }
    if (T.any_upml) T.upml.assign(n * TAB_UPML * 4, 0.f);
    if (T.any_ade) T.ade.assign(n * TAB_ADE * 4, 0.f);
    if (T.adex_orders) {
        T.adex.assign((size_t)T.adex_orders * n * TAB_ADE * 4, 0.f);
        for (int o = 0; o < T.adex_orders; ++o)
            for (size_t k = 0; k < n; ++k)
                std::memcpy(&T.adex[((size_t)o * n + k) * TAB_ADE * 4], tuples[k].ax[o], sizeof(tuples[k].ax[o]));
    }
    for (size_t k = 0; k < n; ++k) {
        const HalfTuple& t = tuples[k];
        float* m = &T.main[k * TAB_MAIN * 4];
        for (int i = 0; i < 6; ++i) m[i] = t.c[i];
        std::memcpy(&m[6], &t.flags, 4);
        if (T.any_upml) std::memcpy(&T.upml[k * TAB_UPML * 4], t.u, sizeof(t.u));
        if (T.any_ade) std::memcpy(&T.ade[k * TAB_ADE * 4], t.a, sizeof(t.a));
        float* x = &T.exc[k * TAB_EXC * 4];
        for (int i = 0; i < 3; ++i) x[i] = t.x[i];
        std::memcpy(&x[4], t.xd, sizeof(t.xd));
    }
}

int alloc_index(HalfTables& T, size_t bytes, bool try_pinned) {
    T.idx_bytes = bytes;
    if (try_pinned && cudaMallocHost(reinterpret_cast<void**>(&T.idx), bytes) == cudaSuccess) {
        T.pinned = true;
    } else {
        cudaGetLastError();
        T.idx = static_cast<uint8_t*>(std::malloc(bytes));
        T.pinned = false;
        if (!T.idx) {
            set_error("host allocation of a tuple index failed");
            return FDTD_ERR_NOMEM;
        }
    }
    std::memset(T.idx, 0, bytes);
    return FDTD_OK;
}

int compress_impl(const fdtd_op_desc* d, int mode, int want_rot, fdtd_cop_s* c) {
    for (int a = 0; a < 3; ++a) {
        if (d->num_lines[a] < 2) {
            set_error("every axis needs at least two lines");
            return FDTD_ERR_ARG;
        }
        c->N0[a] = d->num_lines[a];
    }
    c->rot = choose_rotation(c->N0, want_rot);
    for (int a = 0; a < 3; ++a) c->N[a] = c->N0[(a + c->rot) % 3];
    if (!d->vv || !d->vi || !d->ii || !d->iv) {
        set_error("coefficient arrays missing");
        return FDTD_ERR_ARG;
    }
    if ((d->volt_count || d->curr_count) && (!d->signal_length || !d->signal_volt || !d->signal_curr)) {
        set_error("excitation points without an excitation signal");
        return FDTD_ERR_ARG;
    }
    const bool have_lines = d->lines[0] && d->lines[1] && d->lines[2] && d->unit > 0;
    if (mode == 2 && !have_lines) {
        set_error("factorized compression needs the mesh lines in the operator description");
        return FDTD_ERR_ARG;
    }
    c->dT = d->dT;
    Plan P;
    P.d = d;
    P.rot = c->rot;
    for (int a = 0; a < 3; ++a) {
        P.N[a] = c->N0[a];
        P.D[a] = c->N[a];
    }
    const uint32_t Nx = P.N[0], Ny = P.N[1], Nz = P.N[2];        // reference axes
    const uint32_t Dx = P.D[0], Dy = P.D[1], Dz = P.D[2];        // device axes
    P.NN = (size_t)Nx * Ny * Nz;
    P.geo = (mode == 2) || (mode == 0 && have_lines && !mesh_uniform(d));
    c->geo = P.geo;
    // per-axis arrays are laid out in device axis order; device axis a is
    // reference axis (a + rot) % 3
    if (P.geo) {
        const size_t tot = (size_t)Nx + Ny + Nz;
        c->geom.assign(4 * tot, 0.f);
        size_t off = 0;
        for (int da = 0; da < 3; ++da) {
            const int a = (da + P.rot) % 3;
            const uint32_t N = P.N[a];
            for (uint32_t i = 0; i < N; ++i) {
                const double m = edge_len(d->lines[a], N, i, false, d->unit);
                const double du = edge_len(d->lines[a], N, i, true, d->unit);
                c->geom[0 * tot + off + i] = (float)m;
                c->geom[1 * tot + off + i] = (float)(1.0 / du);
                c->geom[2 * tot + off + i] = (float)du;
                c->geom[3 * tot + off + i] = (float)(1.0 / m);
            }
            for (int k = 0; k < 4; ++k) P.gf[k][a] = &c->geom[k * tot + off];
            off += N;
        }
    }
    if (have_lines) {  // Operator::GetEdgeLength per axis, main and dual, for field dumps
        const size_t tot = (size_t)Nx + Ny + Nz;
        c->edges.assign(2 * tot, 0.0);
        size_t off = 0;
        for (int da = 0; da < 3; ++da) {
            const int a = (da + P.rot) % 3;
            for (uint32_t i = 0; i < P.N[a]; ++i) {
                c->edges[off + i] = edge_len(d->lines[a], P.N[a], i, false, d->unit);
                c->edges[tot + off + i] = edge_len(d->lines[a], P.N[a], i, true, d->unit);
            }
            off += P.N[a];
        }
    }
    int rc = prepare(d, P);
    if (rc) return rc;

    // per x-plane dedup in parallel, then a sequential global merge
    std::vector<std::vector<HalfTuple>> pt[2];
    std::vector<std::vector<uint32_t>> pl[2];
    for (int h = 0; h < 2; ++h) {
        pt[h].resize(Dx);
        pl[h].resize(Dx);
    }
    std::vector<uint32_t> cnt_u(Dx, 0), cnt_a(Dx, 0);
    // device plane x, row y, lane z -> the reference node
    const int ax = (0 + P.rot) % 3, ay = (1 + P.rot) % 3, az = (2 + P.rot) % 3;
    auto worker = [&](uint32_t x) {
        for (int h = 0; h < 2; ++h) {
            TupleMap local = make_map(P.key_bytes);
            std::vector<HalfTuple>& tv = pt[h][x];
            std::vector<uint32_t>& lv = pl[h][x];
            lv.resize((size_t)Dy * Dz);
            HalfTuple t{}, last{};  // value-initialized: bytes past the compared key stay zero
            uint32_t last_id = UINT32_MAX;
            uint32_t o[3];
            o[ax] = x;
            for (uint32_t y = 0; y < Dy; ++y)
                for (uint32_t z = 0; z < Dz; ++z) {
                    o[ay] = y;
                    o[az] = z;
                    const size_t gi = ((size_t)o[0] * Ny + o[1]) * Nz + o[2];
                    make_tuple(P, h, o[0], o[1], o[2], gi, t);
                    if (h == 0) {
                        if (t.flags & TF_UPML) cnt_u[x]++;
                        bool a = !P.ade.empty() && P.ade[gi] >= 0;
                        for (int o = 0; o < kExtraOrders; ++o) a = a || (!P.adex[o].empty() && P.adex[o][gi] >= 0);
                        if (a) cnt_a[x]++;
                    }
                    uint32_t id;
                    if (last_id != UINT32_MAX && std::memcmp(&t, &last, P.key_bytes) == 0) {
                        id = last_id;
                    } else {
                        auto it = local.find(t);
                        if (it == local.end()) {
                            id = (uint32_t)tv.size();
                            local.emplace(t, id);
                            tv.push_back(t);
                        } else {
                            id = it->second;
                        }
                        last = t;
                        last_id = id;
                    }
                    lv[(size_t)y * Dz + z] = id;
                }
        }
    };
    {
        std::atomic<uint32_t> next{0};
        std::vector<std::thread> pool;
        const int nt = std::max(1, std::min<int>((int)std::thread::hardware_concurrency(), (int)Dx));
        for (int t = 0; t < nt; ++t)
            pool.emplace_back([&] {
                for (;;) {
                    const uint32_t x = next.fetch_add(1);
                    if (x >= Dx) break;
                    worker(x);
                }
            });
        for (auto& th : pool) th.join();
    }
    int ndev = 0;
    const bool try_pinned = cudaGetDeviceCount(&ndev) == cudaSuccess && ndev > 0;
    if (!try_pinned) cudaGetLastError();
    c->Nzp = (int)((Dz + 31) / 32 * 32);
    c->comp = (long long)Dx * Dy * c->Nzp;
    std::vector<uint32_t> node_e;  // E tuple per node, for the trim test
    node_e.resize(P.NN);
    std::vector<HalfTuple> all[2];
    for (int h = 0; h < 2; ++h) {
        TupleMap global = make_map(P.key_bytes);
        std::vector<HalfTuple>& tuples = all[h];
        std::vector<std::vector<uint32_t>> remap(Dx);
        for (uint32_t x = 0; x < Dx; ++x) {
            remap[x].resize(pt[h][x].size());
            for (size_t k = 0; k < pt[h][x].size(); ++k) {
                auto it = global.find(pt[h][x][k]);
                if (it == global.end()) {
                    const uint32_t id = (uint32_t)tuples.size();
                    global.emplace(pt[h][x][k], id);
                    tuples.push_back(pt[h][x][k]);
                    remap[x][k] = id;
                } else {
                    remap[x][k] = it->second;
                }
            }
            std::vector<HalfTuple>().swap(pt[h][x]);
        }
        if (P.geo) {  // factorized mode: merge the tuples that differ by rounding variants only
            std::vector<uint64_t> uses(tuples.size(), 0);
            for (uint32_t x = 0; x < Dx; ++x)
                for (uint32_t lid : pl[h][x]) uses[remap[x][lid]]++;
            const std::vector<uint32_t> newid = snap_tuples(tuples, uses, P.key_bytes);
            for (uint32_t x = 0; x < Dx; ++x)
                for (uint32_t& id : remap[x]) id = newid[id];
        }
        HalfTables& T = h ? c->H : c->E;
        T.idx16 = tuples.size() <= 65536;
        const size_t ib = T.idx16 ? 2 : 4;
        if ((rc = alloc_index(T, (size_t)c->comp * ib, try_pinned))) return rc;
        for (uint32_t x = 0; x < Dx; ++x) {
            const std::vector<uint32_t>& lv = pl[h][x];
            for (uint32_t y = 0; y < Dy; ++y) {
                const size_t src = (size_t)y * Dz;
                const size_t dst = ((size_t)x * Dy + y) * c->Nzp;
                for (uint32_t z = 0; z < Dz; ++z) {
                    const uint32_t id = remap[x][lv[src + z]];
                    if (T.idx16)
                        reinterpret_cast<uint16_t*>(T.idx)[dst + z] = (uint16_t)id;
                    else
                        reinterpret_cast<uint32_t*>(T.idx)[dst + z] = id;
                    if (h == 0) node_e[((size_t)x * Dy + y) * Dz + z] = id;
                }
            }
            std::vector<uint32_t>().swap(pl[h][x]);
        }
        pack(tuples, T);
    }
    for (uint32_t x = 0; x < Dx; ++x) {
        c->upml_nodes += cnt_u[x];
        c->ade_nodes += cnt_a[x];
    }
    // An axis' last line is inert for the voltage update when every node on it
    // has only PEC voltage edges (vv = vi = 0), no ADE / excitation and, in
    // UPML slabs, vvp = vvfo = 0: starting from zero its voltages stay zero.
    {
        std::vector<uint8_t> inert(all[0].size());
        for (size_t k = 0; k < all[0].size(); ++k) {
            const HalfTuple& t = all[0][k];
            bool z = true;
            for (int n = 0; n < 6; ++n) z = z && t.c[n] == 0.f;
            if (t.flags & (TF_ADE | TF_ADEX_ALL | TF_EXC)) z = false;
            if (t.flags & TF_UPML)
                for (int n = 0; n < 6; ++n) z = z && t.u[n] == 0.f;
            inert[k] = z;
        }
        for (int a = 0; a < 3; ++a) {
            bool allz = true;
            uint32_t pos[3];
            const int b = (a + 1) % 3, cc = (a + 2) % 3;
            pos[a] = P.D[a] - 1;
            for (pos[b] = 0; pos[b] < P.D[b] && allz; ++pos[b])
                for (pos[cc] = 0; pos[cc] < P.D[cc] && allz; ++pos[cc])
                    allz = inert[node_e[((size_t)pos[0] * Dy + pos[1]) * Dz + pos[2]]] != 0;
            c->trim_e[a] = allz;
        }
    }
    // inner box outside of which the UPML slabs lie (slabs touching a face)
    {
        int lo[3], hi[3];  // reference axes
        for (int a = 0; a < 3; ++a) {
            lo[a] = 0;
            hi[a] = (int)P.N[a] - 1;
        }
        for (uint32_t k = 0; k < d->num_upml; ++k) {
            const fdtd_upml_desc& u = d->upml[k];
            for (int a = 0; a < 3; ++a) {
                if (u.num_lines[a] == P.N[a]) continue;
                if (u.start[a] == 0) lo[a] = std::max(lo[a], (int)u.num_lines[a]);
                if (u.start[a] + u.num_lines[a] == P.N[a]) hi[a] = std::min(hi[a], (int)u.start[a] - 1);
            }
        }
        for (int da = 0; da < 3; ++da) {
            c->inner_lo[da] = lo[(da + P.rot) % 3];
            c->inner_hi[da] = hi[(da + P.rot) % 3];
        }
    }
    c->sig_len = d->signal_length;
    c->sig_period = d->signal_period_ts;
    if (d->signal_length) {
        c->sigV.assign(d->signal_volt, d->signal_volt + d->signal_length);
        c->sigC.assign(d->signal_curr, d->signal_curr + d->signal_length);
    }
    // Mur faces.  The engine applies a face after the node updates of its
    // voltage step, so a face must not meet what the reference applies
    // between its post-update and apply hooks (Lorentz/Drude on the face or
    // its neighbour line, an excitation on the neighbour line); an
    // excitation on the face line itself is added after the face is set,
    // as the reference does.
    for (uint32_t f = 0; f < d->num_mur; ++f) {
        const fdtd_mur_desc& m = d->mur[f];
        if (m.ny < 0 || m.ny > 2 || m.line >= P.N[m.ny] || m.shift >= P.N[m.ny] ||
            m.n_p != P.N[(m.ny + 1) % 3] || m.n_pp != P.N[(m.ny + 2) % 3]) {
            set_error("Mur face descriptor does not match the grid");
            return FDTD_ERR_ARG;
        }
        for (uint32_t o = 0; o < d->num_ade_orders; ++o)
            for (uint32_t i = 0; i < d->ade[o].count; ++i) {
                const uint32_t q = d->ade[o].pos[m.ny][i];
                if (q == m.line || q == m.shift) {
                    set_error("a Lorentz/Drude material touches a Mur boundary (or the line next to it): not provided");
                    return FDTD_ERR_UNSUPPORTED;
                }
            }
        for (uint32_t i = 0; i < d->volt_count; ++i)
            if (d->volt_index[m.ny][i] == m.shift && d->volt_dir[i] != m.ny) {
                set_error("an excitation on the line next to a Mur boundary is not provided");
                return FDTD_ERR_UNSUPPORTED;
            }
        MurFace M;
        // device axis of the face normal; its (nyP, nyPP) layout is unchanged
        // by a cyclic relabelling
        M.ny = (m.ny - P.rot + 3) % 3;
        M.top = m.top;
        M.line = m.line;
        M.shift = m.shift;
        M.n[0] = m.n_p;
        M.n[1] = m.n_pp;
        M.cp.assign(m.coef_p, m.coef_p + (size_t)m.n_p * m.n_pp);
        M.cpp.assign(m.coef_pp, m.coef_pp + (size_t)m.n_p * m.n_pp);
        M.start_ts = m.start_ts;
        c->mur.push_back(std::move(M));
        // a top face's line may stay trimmed from the voltage kernel: the
        // post-update reads the inert line as the zero the update leaves there
    }
    // Lumped RLC edges.  The engine applies them in a pass after the
    // voltage kernel (and the Mur post-update); the reference applies them
    // before the Lorentz/Drude apply and the excitation, which the voltage
    // kernel has already done -- so an RLC edge must not carry either.
    if (d->rlc && d->rlc->count) {
        const fdtd_rlc_desc& r = *d->rlc;
        std::vector<uint64_t> keys(r.count);
        for (uint32_t k = 0; k < r.count; ++k) {
            const int n = r.dir[k];
            if (n < 0 || n > 2 || r.pos[0][k] >= P.N[0] || r.pos[1][k] >= P.N[1] || r.pos[2][k] >= P.N[2]) {
                set_error("lumped RLC edge outside the grid");
                return FDTD_ERR_ARG;
            }
            keys[k] = (((uint64_t)r.pos[0][k] * P.N[1] + r.pos[1][k]) * P.N[2] + r.pos[2][k]) * 3 + n;
        }
        std::vector<uint64_t> sorted = keys;
        std::sort(sorted.begin(), sorted.end());
        if (std::adjacent_find(sorted.begin(), sorted.end()) != sorted.end()) {
            set_error("two lumped RLC elements share an edge: not provided");
            return FDTD_ERR_UNSUPPORTED;
        }
        auto has = [&](uint32_t x, uint32_t y, uint32_t z, int n) {
            const uint64_t key = (((uint64_t)x * P.N[1] + y) * P.N[2] + z) * 3 + n;
            return std::binary_search(sorted.begin(), sorted.end(), key);
        };
        for (uint32_t o = 0; o < d->num_ade_orders; ++o) {
            const fdtd_ade_desc& a = d->ade[o];
            if (!a.volt_on) continue;
            for (uint32_t i = 0; i < a.count; ++i)
                for (int n = 0; n < 3; ++n)
                    if (has(a.pos[0][i], a.pos[1][i], a.pos[2][i], n)) {
                        set_error("a lumped RLC element inside a Lorentz/Drude material: not provided");
                        return FDTD_ERR_UNSUPPORTED;
                    }
        }
        for (uint32_t i = 0; i < d->volt_count; ++i)
            if (has(d->volt_index[0][i], d->volt_index[1][i], d->volt_index[2][i], d->volt_dir[i])) {
                set_error("a voltage excitation on a lumped RLC edge: not provided");
                return FDTD_ERR_UNSUPPORTED;
            }
        // openEMS turns an unset (negative) R, L or C into NaN
        // (operator_ext_lumpedRLC.cpp:188-196); a series element without
        // all three, or a parallel one with L but no R, then has NaN
        // coefficients (:271-273, :307), and its run would turn every
        // field to NaN.  Refused here, before a timestep is spent.
        for (uint32_t k = 0; k < r.count; ++k) {
            const float v[9] = {r.ilv[k], r.i2v[k], r.vv2[k], r.vj1[k], r.vj2[k],
                                r.vvd[k], r.ib0[k], r.b1[k], r.b2[k]};
            for (float x : v)
                if (!std::isfinite(x)) {
                    set_error("a lumped RLC element has non-finite coefficients (openEMS turns an unset R, L or C "
                              "into NaN: a series element needs all three, a parallel one with an L needs its R)");
                    return FDTD_ERR_ARG;
                }
        }
        RlcList& q = c->rlc;  // in device axes
        for (int a = 0; a < 3; ++a) q.pos[a].assign(r.pos[(a + P.rot) % 3], r.pos[(a + P.rot) % 3] + r.count);
        q.dir.resize(r.count);
        for (uint32_t k = 0; k < r.count; ++k) q.dir[k] = (r.dir[k] - P.rot + 3) % 3;
        q.ilv.assign(r.ilv, r.ilv + r.count);
        q.i2v.assign(r.i2v, r.i2v + r.count);
        q.vv2.assign(r.vv2, r.vv2 + r.count);
        q.vj1.assign(r.vj1, r.vj1 + r.count);
        q.vj2.assign(r.vj2, r.vj2 + r.count);
        q.vvd.assign(r.vvd, r.vvd + r.count);
        q.ib0.assign(r.ib0, r.ib0 + r.count);
        q.b1.assign(r.b1, r.b1 + r.count);
        q.b2.assign(r.b2, r.b2 + r.count);
        for (uint32_t k = 0; k < r.count; ++k)
            for (int a = 0; a < 3; ++a)
                if (q.pos[a][k] == c->N[a] - 1) c->trim_e[a] = false;
    }
    return FDTD_OK;
}

}  // namespace
}  // namespace wipems

using namespace wipems;

extern "C" {

int fdtd_compress_rot(const fdtd_op_desc* desc, int mode, int rotation, fdtd_cop_t* out) {
    if (!desc || !out || mode < 0 || mode > 2 || rotation < -1 || rotation > 2) {
        set_error("fdtd_compress: invalid argument");
        return FDTD_ERR_ARG;
    }
    fdtd_cop_s* c = new (std::nothrow) fdtd_cop_s();
    if (!c) return FDTD_ERR_NOMEM;
    int rc;
    try {
        rc = compress_impl(desc, mode, rotation, c);
    } catch (const std::bad_alloc&) {
        set_error("fdtd_compress: host allocation failed");
        rc = FDTD_ERR_NOMEM;
    }
    if (rc != FDTD_OK) {
        delete c;
        return rc;
    }
    *out = c;
    return FDTD_OK;
}

int fdtd_compress_ex(const fdtd_op_desc* desc, int mode, fdtd_cop_t* out) {
    return fdtd_compress_rot(desc, mode, -1, out);
}

int fdtd_compress(const fdtd_op_desc* desc, fdtd_cop_t* out) { return fdtd_compress_ex(desc, 0, out); }

int fdtd_cop_destroy(fdtd_cop_t c) {
    delete c;
    return FDTD_OK;
}

int fdtd_cop_get_info(fdtd_cop_t c, fdtd_cop_info* info) {
    if (!c || !info) return FDTD_ERR_ARG;
    std::memset(info, 0, sizeof(*info));
    for (int a = 0; a < 3; ++a) {
        info->num_lines[a] = c->N0[a];
        info->device_lines[a] = c->N[a];
        info->trim_e[a] = c->trim_e[a] ? 1 : 0;
    }
    info->rotation = c->rot;
    info->num_tuples_e = c->E.num_tuples;
    info->num_tuples_h = c->H.num_tuples;
    info->index_bytes_e = c->E.idx16 ? 2 : 4;
    info->index_bytes_h = c->H.idx16 ? 2 : 4;
    info->padded_nz = (uint32_t)c->Nzp;
    info->num_upml_nodes = c->upml_nodes;
    info->num_ade_nodes = c->ade_nodes;
    info->geometry_factored = c->geo ? 1 : 0;
    size_t tab = 0;
    for (const HalfTables* T : {&c->E, &c->H})
        tab += T->idx_bytes + (T->main.size() + T->upml.size() + T->ade.size() + T->exc.size() + T->adex.size()) * sizeof(float);
    info->host_bytes = tab + c->geom.size() * sizeof(float) + (c->sigV.size() + c->sigC.size()) * sizeof(float);
    info->pinned = (c->E.pinned && c->H.pinned) ? 1 : 0;
    return FDTD_OK;
}

// reference node (x, y, z) -> offset of its device node in the padded index
static size_t dev_index(const fdtd_cop_s* c, const uint32_t o[3]) {
    const int r = c->rot;
    const uint32_t d0 = o[r % 3], d1 = o[(1 + r) % 3], d2 = o[(2 + r) % 3];
    return ((size_t)d0 * c->N[1] + d1) * c->Nzp + d2;
}

int fdtd_cop_expand(fdtd_cop_t c, float* vv, float* vi, float* ii, float* iv, uint32_t* flags_e, uint32_t* flags_h) {
    if (!c) return FDTD_ERR_ARG;
    const uint32_t Nx = c->N0[0], Ny = c->N0[1], Nz = c->N0[2];
    const size_t NN = (size_t)Nx * Ny * Nz;
    const size_t tot = (size_t)Nx + Ny + Nz;
    const size_t off[3] = {0, c->N[0], (size_t)c->N[0] + c->N[1]};  // device axes
    for (uint32_t x = 0; x < Nx; ++x)
        for (uint32_t y = 0; y < Ny; ++y)
            for (uint32_t z = 0; z < Nz; ++z) {
                const uint32_t o[3] = {x, y, z};
                const size_t pi = dev_index(c, o);
                const size_t gi = ((size_t)x * Ny + y) * Nz + z;
                uint32_t pos[3];  // device node
                for (int a = 0; a < 3; ++a) pos[a] = o[(a + c->rot) % 3];
                for (int h = 0; h < 2; ++h) {
                    const HalfTables& T = h ? c->H : c->E;
                    const uint32_t t = T.idx16 ? reinterpret_cast<const uint16_t*>(T.idx)[pi]
                                               : reinterpret_cast<const uint32_t*>(T.idx)[pi];
                    const float* m = &T.main[(size_t)t * TAB_MAIN * 4];
                    float* o1 = h ? ii : vv;
                    float* o2 = h ? iv : vi;
                    for (int k = 0; k < 3; ++k) {  // device component k
                        const int n = (k + c->rot) % 3;
                        if (o1) o1[n * NN + gi] = m[k];
                        float v = m[3 + k];
                        if (c->geo) {
                            // the kernels' float product ((V * g0) * g1) * g2
                            const int kP = (k + 1) % 3, kPP = (k + 2) % 3;
                            const float* g = c->geom.data();
                            const float g0 = g[(h ? 2 : 0) * tot + off[k] + pos[k]];
                            const float g1 = g[(h ? 3 : 1) * tot + off[kP] + pos[kP]];
                            const float g2 = g[(h ? 3 : 1) * tot + off[kPP] + pos[kPP]];
                            v = v * g0;
                            v = v * g1;
                            v = v * g2;
                        }
                        if (o2) o2[n * NN + gi] = v;
                    }
                    uint32_t* f = h ? flags_h : flags_e;
                    if (f) std::memcpy(&f[gi], &m[6], 4);
                }
            }
    return FDTD_OK;
}

// the 9 per-node terms of an extension group (3 kinds x 3 components) of
// tuple t, from the device table tab, into reference layout [9][NN]
static void put9(const fdtd_cop_s* c, const float* tab, size_t gi, size_t NN, bool on, float* out) {
    for (int kind = 0; kind < 3; ++kind)
        for (int k = 0; k < 3; ++k)
            out[(size_t)(3 * kind + (k + c->rot) % 3) * NN + gi] = on ? tab[3 * kind + k] : 0.f;
}

int fdtd_cop_expand_ade(fdtd_cop_t c, int half, int order, float* ade) {
    if (!c || half < 0 || half > 1 || order < 0 || order >= kMaxDispOrder || !ade) return FDTD_ERR_ARG;
    const HalfTables& T = half ? c->H : c->E;
    const uint32_t Nx = c->N0[0], Ny = c->N0[1], Nz = c->N0[2];
    const size_t NN = (size_t)Nx * Ny * Nz;
    const uint32_t bit = order == 0 ? TF_ADE : (TF_ADEX << (order - 1));
    const float* tab = order == 0 ? T.ade.data() : T.adex.data() + (size_t)(order - 1) * T.num_tuples * TAB_ADE * 4;
    for (uint32_t x = 0; x < Nx; ++x)
        for (uint32_t y = 0; y < Ny; ++y)
            for (uint32_t z = 0; z < Nz; ++z) {
                const uint32_t o[3] = {x, y, z};
                const size_t pi = dev_index(c, o);
                const size_t gi = ((size_t)x * Ny + y) * Nz + z;
                const uint32_t t = T.idx16 ? reinterpret_cast<const uint16_t*>(T.idx)[pi]
                                           : reinterpret_cast<const uint32_t*>(T.idx)[pi];
                uint32_t flags;
                std::memcpy(&flags, &T.main[(size_t)t * TAB_MAIN * 4 + 6], 4);
                const bool on = (flags & bit) != 0;
                put9(c, on ? tab + (size_t)t * TAB_ADE * 4 : nullptr, gi, NN, on, ade);
            }
    return FDTD_OK;
}

int fdtd_cop_expand_ext(fdtd_cop_t c, int half, float* ade, float* upml) {
    if (!c || half < 0 || half > 1) return FDTD_ERR_ARG;
    const HalfTables& T = half ? c->H : c->E;
    const uint32_t Nx = c->N0[0], Ny = c->N0[1], Nz = c->N0[2];
    const size_t NN = (size_t)Nx * Ny * Nz;
    for (uint32_t x = 0; x < Nx; ++x)
        for (uint32_t y = 0; y < Ny; ++y)
            for (uint32_t z = 0; z < Nz; ++z) {
                const uint32_t o[3] = {x, y, z};
                const size_t pi = dev_index(c, o);
                const size_t gi = ((size_t)x * Ny + y) * Nz + z;
                const uint32_t t = T.idx16 ? reinterpret_cast<const uint16_t*>(T.idx)[pi]
                                           : reinterpret_cast<const uint32_t*>(T.idx)[pi];
                uint32_t flags;
                std::memcpy(&flags, &T.main[(size_t)t * TAB_MAIN * 4 + 6], 4);
                const bool a = (flags & TF_ADE) != 0, u = (flags & TF_UPML) != 0;
                if (ade) put9(c, a ? &T.ade[(size_t)t * TAB_ADE * 4] : nullptr, gi, NN, a, ade);
                if (upml) put9(c, u ? &T.upml[(size_t)t * TAB_UPML * 4] : nullptr, gi, NN, u, upml);
            }
    return FDTD_OK;
}

}  // extern "C"
