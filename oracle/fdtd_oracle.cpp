// ORACLE -- test infrastructure only.  Nothing in the product links or calls
// this file; tests/, __graft_entry__.smoke() and bench.py's CPU-baseline arm
// use it as the checker / the timed CPU reference.
//
// A CPU restatement of openEMS's FP32 time stepping, written to follow the
// reference's own loops and hook order literally (citations relative to the
// reference project):
//   Engine::UpdateVoltages / UpdateCurrents     FDTD/engine.cpp:108-210
//   Engine::IterateTS + hook order              FDTD/engine.cpp:212-274
//   extension priorities                        extensions/engine_extension.h:21-29
//   SortExtensionByPriority (stable + reverse)  FDTD/engine.cpp:85-96
//   Engine_Ext_UPML pre/post flux swap          extensions/engine_ext_upml.cpp:57-239
//   Engine_Ext_LorentzMaterial pre-updates      extensions/engine_ext_lorentzmaterial.cpp:79-173
//   Engine_Ext_Dispersive::Apply2*              extensions/engine_ext_dispersive.cpp:76-132
//   Engine_Ext_Excitation::Apply2*              extensions/engine_ext_excitation.cpp:33-99
//   Engine_Ext_Mur_ABC pre/post/apply           extensions/engine_ext_mur_abc.cpp:84-164
//   Engine_Ext_LumpedRLC pre/apply              extensions/engine_ext_lumpedRLC.cpp:83-145
//   Engine_Interface_FDTD::CalcVoltageIntegral  FDTD/engine_interface_fdtd.cpp:200-226
//   ProcessCurrent::CalcIntegral (float acc.)   Common/processcurrent.cpp:93-168
//   Engine_Interface_FDTD::CalcFastEnergy       FDTD/engine_interface_fdtd.cpp:292-337
//   ProcessFieldProbe (E / H at a point)        Common/processfieldprobe.cpp:79-92
// and, as the timed CPU baseline, the reference's default engine family:
//   Engine_SSE_Compressed::UpdateVoltages/Currents  FDTD/engine_sse_compressed.cpp:48-263
//     (z-interleaved f4 layout engine_sse.h:36-44, per-vector index
//      operator_sse_compressed.cpp:120-176)
//   Engine_Multithread x-slab workers + barriers    FDTD/engine_multithread.cpp:308-400
//   AssignJobs2Threads                              tools/useful.cpp:45-75
// Compiled with -ffp-contract=off so no product/sum pair is fused into an FMA
// (the reference's x86-64 build has no FMA contraction).
//
// Parity pinning: the reference cannot be built here (it needs CSXCAD,
// fparser, TinyXML, HDF5, Boost, VTK) and ships no golden vectors; this
// restatement is pinned by the closed-form and physics known-answer tests in
// tests/ (excitation signal, Courant timestep, PEC-cavity resonances within
// the TESTSUITE/combinedtests/cavity.m limits) and by the agreement of its
// two engine variants (basic vs SSE-compressed, bitwise, as the reference's
// TESTSUITE/enginetests/cavity.m demands of its own engines).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "../include/wipems_fdtd.h"

namespace {

constexpr double kEps0 = 8.85418781762e-12;
constexpr double kMue0 = 1.256637062e-6;

struct Probe {
    fdtd_probe_desc d;
};

// ------------------------------------------------------------ basic engine
struct BasicEngine {
    uint32_t N[3];
    size_t NN;
    const fdtd_op_desc* op;
    std::vector<float> volt, curr;
    unsigned numTS = 0;
    // UPML state per slab
    std::vector<std::vector<float>> vflux, cflux;
    // ADE state per order
    std::vector<std::vector<float>> vADE, vLor, cADE, cLor;
    // Mur ABC buffers per face (m_volt_nyP / m_volt_nyPP)
    std::vector<std::vector<float>> murP, murPP;
    // lumped RLC state (v_Il, v_Vdn[3], v_Jn[3]), rotated like the reference's pointers
    std::vector<float> rlcIl, rlcVd[3], rlcJ[3];

    explicit BasicEngine(const fdtd_op_desc* d) : op(d) {
        for (int n = 0; n < 3; ++n) N[n] = d->num_lines[n];
        NN = (size_t)N[0] * N[1] * N[2];
        volt.assign(3 * NN, 0.f);
        curr.assign(3 * NN, 0.f);
        for (uint32_t s = 0; s < d->num_upml; ++s) {
            const fdtd_upml_desc& u = d->upml[s];
            size_t nloc = 3 * (size_t)u.num_lines[0] * u.num_lines[1] * u.num_lines[2];
            vflux.emplace_back(nloc, 0.f);
            cflux.emplace_back(nloc, 0.f);
        }
        for (uint32_t f = 0; f < d->num_mur; ++f) {
            murP.emplace_back((size_t)d->mur[f].n_p * d->mur[f].n_pp, 0.f);
            murPP.emplace_back((size_t)d->mur[f].n_p * d->mur[f].n_pp, 0.f);
        }
        if (d->rlc && d->rlc->count) {
            rlcIl.assign(d->rlc->count, 0.f);
            for (int k = 0; k < 3; ++k) {
                rlcVd[k].assign(d->rlc->count, 0.f);
                rlcJ[k].assign(d->rlc->count, 0.f);
            }
        }
        for (uint32_t o = 0; o < d->num_ade_orders; ++o) {
            size_t c = 3 * (size_t)d->ade[o].count;
            vADE.emplace_back(d->ade[o].volt_on ? c : 0, 0.f);
            vLor.emplace_back(d->ade[o].volt_lor_on ? c : 0, 0.f);
            cADE.emplace_back(d->ade[o].curr_on ? c : 0, 0.f);
            cLor.emplace_back(d->ade[o].curr_lor_on ? c : 0, 0.f);
        }
    }
    size_t at(int n, uint32_t x, uint32_t y, uint32_t z) const {
        return (size_t)n * NN + ((size_t)x * N[1] + y) * N[2] + z;
    }
    float& V(int n, uint32_t x, uint32_t y, uint32_t z) { return volt[at(n, x, y, z)]; }
    float& I(int n, uint32_t x, uint32_t y, uint32_t z) { return curr[at(n, x, y, z)]; }
    float cvv(int n, uint32_t x, uint32_t y, uint32_t z) const { return op->vv[at(n, x, y, z)]; }
    float cvi(int n, uint32_t x, uint32_t y, uint32_t z) const { return op->vi[at(n, x, y, z)]; }
    float cii(int n, uint32_t x, uint32_t y, uint32_t z) const { return op->ii[at(n, x, y, z)]; }
    float civ(int n, uint32_t x, uint32_t y, uint32_t z) const { return op->iv[at(n, x, y, z)]; }

    void update_voltages(uint32_t startX, uint32_t numX) {  // engine.cpp:108-161
        uint32_t pos[3];
        bool shift[3];
        pos[0] = startX;
        for (uint32_t posX = 0; posX < numX; ++posX) {
            shift[0] = pos[0];
            for (pos[1] = 0; pos[1] < N[1]; ++pos[1]) {
                shift[1] = pos[1];
                for (pos[2] = 0; pos[2] < N[2]; ++pos[2]) {
                    shift[2] = pos[2];
                    uint32_t x = pos[0], y = pos[1], z = pos[2];
                    V(0, x, y, z) *= cvv(0, x, y, z);
                    V(0, x, y, z) += cvi(0, x, y, z) *
                                     (I(2, x, y, z) - I(2, x, y - shift[1], z) - I(1, x, y, z) + I(1, x, y, z - shift[2]));
                    V(1, x, y, z) *= cvv(1, x, y, z);
                    V(1, x, y, z) += cvi(1, x, y, z) *
                                     (I(0, x, y, z) - I(0, x, y, z - shift[2]) - I(2, x, y, z) + I(2, x - shift[0], y, z));
                    V(2, x, y, z) *= cvv(2, x, y, z);
                    V(2, x, y, z) += cvi(2, x, y, z) *
                                     (I(1, x, y, z) - I(1, x - shift[0], y, z) - I(0, x, y, z) + I(0, x, y - shift[1], z));
                }
            }
            ++pos[0];
        }
    }
    void update_currents(uint32_t startX, uint32_t numX) {  // engine.cpp:163-210
        uint32_t pos[3];
        pos[0] = startX;
        for (uint32_t posX = 0; posX < numX; ++posX) {
            for (pos[1] = 0; pos[1] < N[1] - 1; ++pos[1]) {
                for (pos[2] = 0; pos[2] < N[2] - 1; ++pos[2]) {
                    uint32_t x = pos[0], y = pos[1], z = pos[2];
                    I(0, x, y, z) *= cii(0, x, y, z);
                    I(0, x, y, z) += civ(0, x, y, z) *
                                     (V(2, x, y, z) - V(2, x, y + 1, z) - V(1, x, y, z) + V(1, x, y, z + 1));
                    I(1, x, y, z) *= cii(1, x, y, z);
                    I(1, x, y, z) += civ(1, x, y, z) *
                                     (V(0, x, y, z) - V(0, x, y, z + 1) - V(2, x, y, z) + V(2, x + 1, y, z));
                    I(2, x, y, z) *= cii(2, x, y, z);
                    I(2, x, y, z) += civ(2, x, y, z) *
                                     (V(1, x, y, z) - V(1, x + 1, y, z) - V(0, x, y, z) + V(0, x, y + 1, z));
                }
            }
            ++pos[0];
        }
    }

    // ---- UPML (engine_ext_upml.cpp)
    template <bool VOLT, bool PRE>
    void upml(uint32_t s) {
        const fdtd_upml_desc& u = op->upml[s];
        const size_t nloc = (size_t)u.num_lines[0] * u.num_lines[1] * u.num_lines[2];
        std::vector<float>& flux = VOLT ? vflux[s] : cflux[s];
        const float* c1 = VOLT ? u.vv : u.ii;
        const float* fo = VOLT ? u.vvfo : u.iifo;
        const float* fn = VOLT ? u.vvfn : u.iifn;
        for (uint32_t lx = 0; lx < u.num_lines[0]; ++lx)
            for (uint32_t ly = 0; ly < u.num_lines[1]; ++ly)
                for (uint32_t lz = 0; lz < u.num_lines[2]; ++lz) {
                    size_t li = ((size_t)lx * u.num_lines[1] + ly) * u.num_lines[2] + lz;
                    uint32_t x = lx + u.start[0], y = ly + u.start[1], z = lz + u.start[2];
                    for (int n = 0; n < 3; ++n) {
                        float& f = flux[n * nloc + li];
                        float& fld = VOLT ? V(n, x, y, z) : I(n, x, y, z);
                        float f_help;
                        if (PRE) {
                            f_help = c1[n * nloc + li] * fld - fo[n * nloc + li] * f;
                            fld = f;
                            f = f_help;
                        } else {
                            f_help = f;
                            f = fld;
                            fld = f_help + fn[n * nloc + li] * f;
                        }
                    }
                }
    }

    // ---- Mur ABC (engine_ext_mur_abc.cpp:84-164), V(n, x, y, z) -> float&.
    // stage 0: DoPreVoltageUpdates (faces in insertion order), 1:
    // DoPostVoltageUpdates, 2: Apply2Voltages (both in reverse insertion
    // order: the sorted extension list holds equal priorities reversed).
    template <class Acc>
    void mur(int stage, unsigned ts, Acc&& Vf) {
        const uint32_t nf = op->num_mur;
        for (uint32_t k = 0; k < nf; ++k) {
            const uint32_t f = stage == 0 ? k : nf - 1 - k;
            const fdtd_mur_desc& m = op->mur[f];
            if (ts < m.start_ts) continue;  // IsActive
            const int ny = m.ny, nP = (ny + 1) % 3, nPP = (ny + 2) % 3;
            uint32_t pos[3], sh[3];
            pos[ny] = m.line;
            sh[ny] = m.shift;
            for (uint32_t i = 0; i < m.n_p; ++i) {
                pos[nP] = sh[nP] = i;
                for (uint32_t j = 0; j < m.n_pp; ++j) {
                    pos[nPP] = sh[nPP] = j;
                    const size_t k2 = (size_t)i * m.n_pp + j;
                    float& bp = murP[f][k2];
                    float& bpp = murPP[f][k2];
                    if (stage == 0) {
                        bp = Vf(nP, sh[0], sh[1], sh[2]) - m.coef_p[k2] * Vf(nP, pos[0], pos[1], pos[2]);
                        bpp = Vf(nPP, sh[0], sh[1], sh[2]) - m.coef_pp[k2] * Vf(nPP, pos[0], pos[1], pos[2]);
                    } else if (stage == 1) {
                        bp += m.coef_p[k2] * Vf(nP, sh[0], sh[1], sh[2]);
                        bpp += m.coef_pp[k2] * Vf(nPP, sh[0], sh[1], sh[2]);
                    } else {
                        Vf(nP, pos[0], pos[1], pos[2]) = bp;
                        Vf(nPP, pos[0], pos[1], pos[2]) = bpp;
                    }
                }
            }
        }
    }

    // ---- lumped RLC (engine_ext_lumpedRLC.cpp:83-145)
    void rlc_pre() {  // DoPreVoltageUpdates: rotate Vd, parallel inductor current
        if (!op->rlc || !op->rlc->count) return;
        const fdtd_rlc_desc& r = *op->rlc;
        std::swap(rlcVd[2], rlcVd[1]);  // Vd[2] <- Vd[1], Vd[1] <- Vd[0], Vd[0] <- old Vd[2]
        std::swap(rlcVd[1], rlcVd[0]);
        for (uint32_t k = 0; k < r.count; ++k) rlcIl[k] += r.i2v[k] * r.ilv[k] * rlcVd[1][k];
    }
    template <class Acc>
    void rlc_apply(Acc&& Vf) {  // Apply2Voltages
        if (!op->rlc || !op->rlc->count) return;
        const fdtd_rlc_desc& r = *op->rlc;
        std::swap(rlcJ[2], rlcJ[1]);
        std::swap(rlcJ[1], rlcJ[0]);
        for (uint32_t k = 0; k < r.count; ++k) rlcVd[0][k] = Vf(r.dir[k], r.pos[0][k], r.pos[1][k], r.pos[2][k]);
        for (uint32_t k = 0; k < r.count; ++k) {
            rlcVd[0][k] = r.vvd[k] * (rlcVd[0][k] - rlcIl[k] + r.vv2[k] * rlcVd[2][k] + r.vj1[k] * rlcJ[1][k] +
                                      r.vj2[k] * rlcJ[2][k]);
            rlcJ[0][k] = r.ib0[k] * (rlcVd[0][k] - rlcVd[2][k]) - (r.b1[k] * r.ib0[k]) * rlcJ[1][k] -
                         (r.b2[k] * r.ib0[k]) * rlcJ[2][k];
        }
        for (uint32_t k = 0; k < r.count; ++k) Vf(r.dir[k], r.pos[0][k], r.pos[1][k], r.pos[2][k]) = rlcVd[0][k];
    }

    // ---- Lorentz / Drude (engine_ext_lorentzmaterial.cpp:79-173)
    template <bool VOLT>
    void ade_pre() {
        for (uint32_t o = 0; o < op->num_ade_orders; ++o) {
            const fdtd_ade_desc& a = op->ade[o];
            if (VOLT ? !a.volt_on : !a.curr_on) continue;
            const float* vint = VOLT ? a.v_int : a.i_int;
            const float* vext = VOLT ? a.v_ext : a.i_ext;
            const float* vlor = VOLT ? a.v_lor : a.i_lor;
            std::vector<float>& A = VOLT ? vADE[o] : cADE[o];
            std::vector<float>& L = VOLT ? vLor[o] : cLor[o];
            bool lor = VOLT ? a.volt_lor_on : a.curr_lor_on;
            const uint32_t c = a.count;
            for (uint32_t i = 0; i < c; ++i) {
                uint32_t x = a.pos[0][i], y = a.pos[1][i], z = a.pos[2][i];
                for (int n = 0; n < 3; ++n) {
                    float fld = VOLT ? V(n, x, y, z) : I(n, x, y, z);
                    if (lor) {
                        L[n * c + i] += vlor[n * c + i] * A[n * c + i];
                        A[n * c + i] *= vint[n * c + i];
                        A[n * c + i] += vext[n * c + i] * (fld - L[n * c + i]);
                    } else {
                        A[n * c + i] *= vint[n * c + i];
                        A[n * c + i] += vext[n * c + i] * fld;
                    }
                }
            }
        }
    }
    template <bool VOLT>
    void ade_apply() {  // engine_ext_dispersive.cpp:76-132
        for (uint32_t o = 0; o < op->num_ade_orders; ++o) {
            const fdtd_ade_desc& a = op->ade[o];
            if (VOLT ? !a.volt_on : !a.curr_on) continue;
            std::vector<float>& A = VOLT ? vADE[o] : cADE[o];
            const uint32_t c = a.count;
            for (uint32_t i = 0; i < c; ++i) {
                uint32_t x = a.pos[0][i], y = a.pos[1][i], z = a.pos[2][i];
                for (int n = 0; n < 3; ++n) {
                    float& fld = VOLT ? V(n, x, y, z) : I(n, x, y, z);
                    fld = fld - A[n * c + i];
                }
            }
        }
    }
    // ---- excitation (engine_ext_excitation.cpp:33-99)
    template <bool VOLT>
    void excite() {
        int numTS_i = (int)numTS;
        unsigned length = op->signal_length;
        int p = numTS_i + 1;
        if (op->signal_period_ts > 0) p = (int)op->signal_period_ts;
        uint32_t cnt = VOLT ? op->volt_count : op->curr_count;
        const float* sig = VOLT ? op->signal_volt : op->signal_curr;
        for (uint32_t n = 0; n < cnt; ++n) {
            int exc_pos = numTS_i - (int)(VOLT ? op->volt_delay[n] : op->curr_delay[n]);
            exc_pos *= (exc_pos > 0);
            exc_pos %= p;
            exc_pos *= (exc_pos < (int)length);
            int ny = VOLT ? op->volt_dir[n] : op->curr_dir[n];
            uint32_t x = (VOLT ? op->volt_index[0] : op->curr_index[0])[n];
            uint32_t y = (VOLT ? op->volt_index[1] : op->curr_index[1])[n];
            uint32_t z = (VOLT ? op->volt_index[2] : op->curr_index[2])[n];
            float amp = VOLT ? op->volt_amp[n] : op->curr_amp[n];
            float& fld = VOLT ? V(ny, x, y, z) : I(ny, x, y, z);
            fld = fld + amp * sig[exc_pos];
        }
    }

    // Engine::IterateTS with the extension list sorted by priority:
    // [UPML slabs (1e6, reverse insertion), lumped RLC, Lorentz, Mur faces
    // (all 0, reverse insertion: the boundaries are added first, then
    // Lorentz, then RLC, openems.cpp:1051-1096), Excitation (-1000)].
    // Pre hooks run in reverse list order, post / apply hooks in list order.
    void iterate(unsigned iterTS) {
        const uint32_t nu = op->num_upml;
        auto Vf = [this](int n, uint32_t x, uint32_t y, uint32_t z) -> float& { return V(n, x, y, z); };
        for (unsigned it = 0; it < iterTS; ++it) {
            // DoPreVoltageUpdates: excitation (none), Mur faces, Lorentz, RLC, UPML slabs
            mur(0, numTS, Vf);
            ade_pre<true>();
            rlc_pre();
            for (uint32_t s = 0; s < nu; ++s) upml<true, true>(s);
            update_voltages(0, N[0]);
            for (uint32_t s = nu; s-- > 0;) upml<true, false>(s);
            mur(1, numTS, Vf);
            rlc_apply(Vf);
            ade_apply<true>();
            mur(2, numTS, Vf);
            excite<true>();

            ade_pre<false>();
            for (uint32_t s = 0; s < nu; ++s) upml<false, true>(s);
            update_currents(0, N[0] - 1);
            for (uint32_t s = nu; s-- > 0;) upml<false, false>(s);
            ade_apply<false>();
            excite<false>();
            ++numTS;
        }
    }

    // Operator::GetEdgeLength (GetDiscDelta x grid delta) from the mesh lines
    double edge_length(int n, uint32_t pos, bool dual) const {
        const double* l = op->lines[n];
        if (!l) return 0.0;
        const uint32_t Nn = N[n];
        auto line = [&](uint32_t p, bool du) -> double {
            if (!du) return l[p];
            if (p < Nn - 1) return 0.5 * (l[p] + l[p + 1]);
            return l[p] + 0.5 * (l[p] - l[p - 1]);
        };
        double d;
        if (!dual)
            d = (pos < Nn - 1) ? line(pos + 1, false) - line(pos, false) : line(pos, false) - line(pos - 1, false);
        else
            d = (pos > 0) ? line(pos, true) - line(pos - 1, true) : line(1, false) - line(0, false);
        return d * op->unit;
    }
    // Engine_Interface_FDTD::GetRawField / GetRawDualField, type 0
    // (engine_interface_fdtd.cpp:257-262, 128-133)
    double raw_field(bool h, int n, const uint32_t* pos) {
        const double value = h ? I(n, pos[0], pos[1], pos[2]) : V(n, pos[0], pos[1], pos[2]);
        const double delta = edge_length(n, pos[n], h);
        if (delta) return value / delta;
        return 0.0;
    }

    double voltage_integral(const uint32_t* start, const uint32_t* stop) {
        if (((start[0] != stop[0]) + (start[1] != stop[1]) + (start[2] != stop[2])) != 1) return 0;
        double result = 0;
        for (int n = 0; n < 3; ++n) {
            if (start[n] < stop[n]) {
                uint32_t pos[3] = {start[0], start[1], start[2]};
                for (; pos[n] < stop[n]; ++pos[n]) result += V(n, pos[0], pos[1], pos[2]);
            } else {
                uint32_t pos[3] = {stop[0], stop[1], stop[2]};
                for (; pos[n] < start[n]; ++pos[n]) result -= V(n, pos[0], pos[1], pos[2]);
            }
        }
        return result;
    }
    double current_integral(const fdtd_probe_desc& p) {
        float current = 0;
        const uint32_t* start = p.start;
        const uint32_t* stop = p.stop;
        const int* si = p.start_inside;
        const int* so = p.stop_inside;
        switch (p.norm_dir) {
            case 0:
                if (so[0] && si[2]) for (uint32_t i = start[1] + 1; i <= stop[1]; ++i) current += I(1, stop[0], i, start[2]);
                if (so[0] && so[1]) for (uint32_t i = start[2] + 1; i <= stop[2]; ++i) current += I(2, stop[0], stop[1], i);
                if (si[0] && so[2]) for (uint32_t i = start[1] + 1; i <= stop[1]; ++i) current -= I(1, start[0], i, stop[2]);
                if (si[0] && si[1]) for (uint32_t i = start[2] + 1; i <= stop[2]; ++i) current -= I(2, start[0], start[1], i);
                break;
            case 1:
                if (si[0] && si[1]) for (uint32_t i = start[2] + 1; i <= stop[2]; ++i) current += I(2, start[0], start[1], i);
                if (so[1] && so[2]) for (uint32_t i = start[0] + 1; i <= stop[0]; ++i) current += I(0, i, stop[1], stop[2]);
                if (so[0] && so[1]) for (uint32_t i = start[2] + 1; i <= stop[2]; ++i) current -= I(2, stop[0], stop[1], i);
                if (si[1] && si[2]) for (uint32_t i = start[0] + 1; i <= stop[0]; ++i) current -= I(0, i, start[1], start[2]);
                break;
            case 2:
                if (si[1] && si[2]) for (uint32_t i = start[0] + 1; i <= stop[0]; ++i) current += I(0, i, start[1], start[2]);
                if (so[0] && si[2]) for (uint32_t i = start[1] + 1; i <= stop[1]; ++i) current += I(1, stop[0], i, start[2]);
                if (so[1] && so[2]) for (uint32_t i = start[0] + 1; i <= stop[0]; ++i) current -= I(0, i, stop[1], stop[2]);
                if (si[0] && so[2]) for (uint32_t i = start[1] + 1; i <= stop[1]; ++i) current -= I(1, start[0], i, stop[2]);
                break;
            default:
                return 0.0;
        }
        return current;
    }
    double fast_energy() {
        double E = 0.0, H = 0.0;
        for (uint32_t x = 0; x < N[0] - 1; ++x)
            for (uint32_t y = 0; y < N[1] - 1; ++y)
                for (uint32_t z = 0; z < N[2] - 1; ++z)
                    for (int n = 0; n < 3; ++n) {
                        E += V(n, x, y, z) * V(n, x, y, z);
                        H += I(n, x, y, z) * I(n, x, y, z);
                    }
        return kEps0 * E + kMue0 * H;
    }
};

// --------------------------------------------- SSE-compressed + x-slab MT
// The timed CPU baseline.  Fields in the z-interleaved f4 layout
// (engine_sse.h:36-44), coefficients deduplicated per f4 vector into an
// index (operator_sse_compressed.cpp:120-176), x-slabs per worker thread
// with barriers after every hook (engine_multithread.cpp:308-400).
typedef float v4sf __attribute__((vector_size(16)));

struct Barrier {
    std::mutex m;
    std::condition_variable cv;
    unsigned count, waiting = 0, gen = 0;
    explicit Barrier(unsigned c) : count(c) {}
    void wait() {
        std::unique_lock<std::mutex> lk(m);
        unsigned g = gen;
        if (++waiting == count) {
            waiting = 0;
            ++gen;
            cv.notify_all();
        } else {
            cv.wait(lk, [&] { return g != gen; });
        }
    }
};

struct SSEEngine {
    uint32_t N[3];
    uint32_t nv;  // numVectors
    const fdtd_op_desc* op;
    std::vector<v4sf> fv, fc;  // [3][Nx][Ny][nv]
    std::vector<uint32_t> index;  // [Nx][Ny][nv]
    std::vector<v4sf> cvv[3], cvi[3], cii[3], civ[3];
    BasicEngine* ext;  // extension state / hooks run through scalar accessors
    unsigned numTS = 0;

    size_t vat(int n, uint32_t x, uint32_t y, uint32_t zv) const {
        return (((size_t)n * N[0] + x) * N[1] + y) * nv + zv;
    }
    float& Vs(int n, uint32_t x, uint32_t y, uint32_t z) {
        return reinterpret_cast<float*>(&fv[vat(n, x, y, z % nv)])[z / nv];
    }
    float& Is(int n, uint32_t x, uint32_t y, uint32_t z) {
        return reinterpret_cast<float*>(&fc[vat(n, x, y, z % nv)])[z / nv];
    }

    explicit SSEEngine(const fdtd_op_desc* d) : op(d), ext(nullptr) {
        for (int n = 0; n < 3; ++n) N[n] = d->num_lines[n];
        nv = (N[2] + 3) / 4;  // ceil(numLines[2]/4) (engine_sse.cpp:43)
        v4sf zero = {0, 0, 0, 0};
        fv.assign(3 * (size_t)N[0] * N[1] * nv, zero);
        fc.assign(3 * (size_t)N[0] * N[1] * nv, zero);
        index.assign((size_t)N[0] * N[1] * nv, 0);
        // CompressOperator: unique 12 x f4 tuples
        struct Key {
            float f[48];
            bool operator<(const Key& o) const { return std::memcmp(f, o.f, sizeof(f)) < 0; }
        };
        std::map<Key, uint32_t> lut;
        size_t NN = (size_t)N[0] * N[1] * N[2];
        for (uint32_t x = 0; x < N[0]; ++x)
            for (uint32_t y = 0; y < N[1]; ++y)
                for (uint32_t zv = 0; zv < nv; ++zv) {
                    Key k;
                    std::memset(&k, 0, sizeof(k));
                    for (int n = 0; n < 3; ++n)
                        for (int l = 0; l < 4; ++l) {
                            uint32_t z = zv + l * nv;
                            if (z >= N[2]) continue;
                            size_t gi = (size_t)n * NN + ((size_t)x * N[1] + y) * N[2] + z;
                            k.f[n * 16 + 0 * 4 + l] = d->vv[gi];
                            k.f[n * 16 + 1 * 4 + l] = d->vi[gi];
                            k.f[n * 16 + 2 * 4 + l] = d->ii[gi];
                            k.f[n * 16 + 3 * 4 + l] = d->iv[gi];
                        }
                    auto it = lut.find(k);
                    uint32_t id;
                    if (it == lut.end()) {
                        id = (uint32_t)cvv[0].size();
                        lut[k] = id;
                        for (int n = 0; n < 3; ++n) {
                            v4sf a, b, c, e;
                            for (int l = 0; l < 4; ++l) {
                                a[l] = k.f[n * 16 + l];
                                b[l] = k.f[n * 16 + 4 + l];
                                c[l] = k.f[n * 16 + 8 + l];
                                e[l] = k.f[n * 16 + 12 + l];
                            }
                            cvv[n].push_back(a);
                            cvi[n].push_back(b);
                            cii[n].push_back(c);
                            civ[n].push_back(e);
                        }
                    } else {
                        id = it->second;
                    }
                    index[((size_t)x * N[1] + y) * nv + zv] = id;
                }
    }

    // engine_sse_compressed.cpp:48-156 (generic lane shift, :107-110)
    void update_voltages(uint32_t startX, uint32_t numX) {
        uint32_t pos[3];
        bool shift[2];
        v4sf temp;
        pos[0] = startX;
        for (uint32_t posX = 0; posX < numX; ++posX) {
            shift[0] = pos[0];
            for (pos[1] = 0; pos[1] < N[1]; ++pos[1]) {
                shift[1] = pos[1];
                const uint32_t x = pos[0], y = pos[1];
                for (pos[2] = 1; pos[2] < nv; ++pos[2]) {
                    const uint32_t z = pos[2];
                    uint32_t id = index[((size_t)x * N[1] + y) * nv + z];
                    fv[vat(0, x, y, z)] *= cvv[0][id];
                    fv[vat(0, x, y, z)] += cvi[0][id] * (fc[vat(2, x, y, z)] - fc[vat(2, x, y - shift[1], z)] -
                                                          fc[vat(1, x, y, z)] + fc[vat(1, x, y, z - 1)]);
                    fv[vat(1, x, y, z)] *= cvv[1][id];
                    fv[vat(1, x, y, z)] += cvi[1][id] * (fc[vat(0, x, y, z)] - fc[vat(0, x, y, z - 1)] -
                                                          fc[vat(2, x, y, z)] + fc[vat(2, x - shift[0], y, z)]);
                    fv[vat(2, x, y, z)] *= cvv[2][id];
                    fv[vat(2, x, y, z)] += cvi[2][id] * (fc[vat(1, x, y, z)] - fc[vat(1, x - shift[0], y, z)] -
                                                          fc[vat(0, x, y, z)] + fc[vat(0, x, y - shift[1], z)]);
                }
                uint32_t id = index[((size_t)x * N[1] + y) * nv + 0];
                const v4sf& l1 = fc[vat(1, x, y, nv - 1)];
                temp[0] = 0; temp[1] = l1[0]; temp[2] = l1[1]; temp[3] = l1[2];
                fv[vat(0, x, y, 0)] *= cvv[0][id];
                fv[vat(0, x, y, 0)] += cvi[0][id] * (fc[vat(2, x, y, 0)] - fc[vat(2, x, y - shift[1], 0)] -
                                                      fc[vat(1, x, y, 0)] + temp);
                const v4sf& l0 = fc[vat(0, x, y, nv - 1)];
                temp[0] = 0; temp[1] = l0[0]; temp[2] = l0[1]; temp[3] = l0[2];
                fv[vat(1, x, y, 0)] *= cvv[1][id];
                fv[vat(1, x, y, 0)] += cvi[1][id] * (fc[vat(0, x, y, 0)] - temp - fc[vat(2, x, y, 0)] +
                                                      fc[vat(2, x - shift[0], y, 0)]);
                fv[vat(2, x, y, 0)] *= cvv[2][id];
                fv[vat(2, x, y, 0)] += cvi[2][id] * (fc[vat(1, x, y, 0)] - fc[vat(1, x - shift[0], y, 0)] -
                                                      fc[vat(0, x, y, 0)] + fc[vat(0, x, y - shift[1], 0)]);
            }
            ++pos[0];
        }
    }
    // engine_sse_compressed.cpp:158-263
    void update_currents(uint32_t startX, uint32_t numX) {
        uint32_t pos[3];
        v4sf temp;
        pos[0] = startX;
        for (uint32_t posX = 0; posX < numX; ++posX) {
            for (pos[1] = 0; pos[1] < N[1] - 1; ++pos[1]) {
                const uint32_t x = pos[0], y = pos[1];
                for (pos[2] = 0; pos[2] < nv - 1; ++pos[2]) {
                    const uint32_t z = pos[2];
                    uint32_t id = index[((size_t)x * N[1] + y) * nv + z];
                    fc[vat(0, x, y, z)] *= cii[0][id];
                    fc[vat(0, x, y, z)] += civ[0][id] * (fv[vat(2, x, y, z)] - fv[vat(2, x, y + 1, z)] -
                                                          fv[vat(1, x, y, z)] + fv[vat(1, x, y, z + 1)]);
                    fc[vat(1, x, y, z)] *= cii[1][id];
                    fc[vat(1, x, y, z)] += civ[1][id] * (fv[vat(0, x, y, z)] - fv[vat(0, x, y, z + 1)] -
                                                          fv[vat(2, x, y, z)] + fv[vat(2, x + 1, y, z)]);
                    fc[vat(2, x, y, z)] *= cii[2][id];
                    fc[vat(2, x, y, z)] += civ[2][id] * (fv[vat(1, x, y, z)] - fv[vat(1, x + 1, y, z)] -
                                                          fv[vat(0, x, y, z)] + fv[vat(0, x, y + 1, z)]);
                }
                const uint32_t z = nv - 1;
                uint32_t id = index[((size_t)x * N[1] + y) * nv + z];
                const v4sf& f1 = fv[vat(1, x, y, 0)];
                temp[0] = f1[1]; temp[1] = f1[2]; temp[2] = f1[3]; temp[3] = 0;
                fc[vat(0, x, y, z)] *= cii[0][id];
                fc[vat(0, x, y, z)] += civ[0][id] * (fv[vat(2, x, y, z)] - fv[vat(2, x, y + 1, z)] -
                                                      fv[vat(1, x, y, z)] + temp);
                const v4sf& f0 = fv[vat(0, x, y, 0)];
                temp[0] = f0[1]; temp[1] = f0[2]; temp[2] = f0[3]; temp[3] = 0;
                fc[vat(1, x, y, z)] *= cii[1][id];
                fc[vat(1, x, y, z)] += civ[1][id] * (fv[vat(0, x, y, z)] - temp - fv[vat(2, x, y, z)] +
                                                      fv[vat(2, x + 1, y, z)]);
                fc[vat(2, x, y, z)] *= cii[2][id];
                fc[vat(2, x, y, z)] += civ[2][id] * (fv[vat(1, x, y, z)] - fv[vat(1, x + 1, y, z)] -
                                                      fv[vat(0, x, y, z)] + fv[vat(0, x, y + 1, z)]);
            }
            ++pos[0];
        }
    }
};

// Extension hooks for the SSE engine go through GetVolt/SetVolt on the
// interleaved layout, exactly as ENG_DISPATCH routes them for Engine::SSE.
struct SSEHooks {
    SSEEngine& s;
    BasicEngine& b;  // provides the extension state arrays and descriptors
    template <bool VOLT>
    float& F(int n, uint32_t x, uint32_t y, uint32_t z) {
        return VOLT ? s.Vs(n, x, y, z) : s.Is(n, x, y, z);
    }
    template <bool VOLT, bool PRE>
    void upml(uint32_t sl, uint32_t x_begin, uint32_t x_count) {
        const fdtd_upml_desc& u = b.op->upml[sl];
        const size_t nloc = (size_t)u.num_lines[0] * u.num_lines[1] * u.num_lines[2];
        std::vector<float>& flux = VOLT ? b.vflux[sl] : b.cflux[sl];
        const float* c1 = VOLT ? u.vv : u.ii;
        const float* fo = VOLT ? u.vvfo : u.iifo;
        const float* fn = VOLT ? u.vvfn : u.iifn;
        for (uint32_t lx = x_begin; lx < x_begin + x_count; ++lx)
            for (uint32_t ly = 0; ly < u.num_lines[1]; ++ly)
                for (uint32_t lz = 0; lz < u.num_lines[2]; ++lz) {
                    size_t li = ((size_t)lx * u.num_lines[1] + ly) * u.num_lines[2] + lz;
                    uint32_t x = lx + u.start[0], y = ly + u.start[1], z = lz + u.start[2];
                    for (int n = 0; n < 3; ++n) {
                        float& f = flux[n * nloc + li];
                        float& fld = F<VOLT>(n, x, y, z);
                        float f_help;
                        if (PRE) {
                            f_help = c1[n * nloc + li] * fld - fo[n * nloc + li] * f;
                            fld = f;
                            f = f_help;
                        } else {
                            f_help = f;
                            f = fld;
                            fld = f_help + fn[n * nloc + li] * f;
                        }
                    }
                }
    }
    template <bool VOLT>
    void ade_pre() {
        for (uint32_t o = 0; o < b.op->num_ade_orders; ++o) {
            const fdtd_ade_desc& a = b.op->ade[o];
            if (VOLT ? !a.volt_on : !a.curr_on) continue;
            const float* vint = VOLT ? a.v_int : a.i_int;
            const float* vext = VOLT ? a.v_ext : a.i_ext;
            const float* vlor = VOLT ? a.v_lor : a.i_lor;
            std::vector<float>& A = VOLT ? b.vADE[o] : b.cADE[o];
            std::vector<float>& L = VOLT ? b.vLor[o] : b.cLor[o];
            bool lor = VOLT ? a.volt_lor_on : a.curr_lor_on;
            const uint32_t c = a.count;
            for (uint32_t i = 0; i < c; ++i)
                for (int n = 0; n < 3; ++n) {
                    float fld = F<VOLT>(n, a.pos[0][i], a.pos[1][i], a.pos[2][i]);
                    if (lor) {
                        L[n * c + i] += vlor[n * c + i] * A[n * c + i];
                        A[n * c + i] *= vint[n * c + i];
                        A[n * c + i] += vext[n * c + i] * (fld - L[n * c + i]);
                    } else {
                        A[n * c + i] *= vint[n * c + i];
                        A[n * c + i] += vext[n * c + i] * fld;
                    }
                }
        }
    }
    template <bool VOLT>
    void ade_apply() {
        for (uint32_t o = 0; o < b.op->num_ade_orders; ++o) {
            const fdtd_ade_desc& a = b.op->ade[o];
            if (VOLT ? !a.volt_on : !a.curr_on) continue;
            std::vector<float>& A = VOLT ? b.vADE[o] : b.cADE[o];
            const uint32_t c = a.count;
            for (uint32_t i = 0; i < c; ++i)
                for (int n = 0; n < 3; ++n) {
                    float& fld = F<VOLT>(n, a.pos[0][i], a.pos[1][i], a.pos[2][i]);
                    fld = fld - A[n * c + i];
                }
        }
    }
    template <bool VOLT>
    void excite(unsigned numTS) {
        const fdtd_op_desc* op = b.op;
        int numTS_i = (int)numTS;
        int p = numTS_i + 1;
        if (op->signal_period_ts > 0) p = (int)op->signal_period_ts;
        uint32_t cnt = VOLT ? op->volt_count : op->curr_count;
        const float* sig = VOLT ? op->signal_volt : op->signal_curr;
        for (uint32_t n = 0; n < cnt; ++n) {
            int exc_pos = numTS_i - (int)(VOLT ? op->volt_delay[n] : op->curr_delay[n]);
            exc_pos *= (exc_pos > 0);
            exc_pos %= p;
            exc_pos *= (exc_pos < (int)op->signal_length);
            int ny = VOLT ? op->volt_dir[n] : op->curr_dir[n];
            float& fld = F<VOLT>(ny, (VOLT ? op->volt_index[0] : op->curr_index[0])[n],
                                 (VOLT ? op->volt_index[1] : op->curr_index[1])[n],
                                 (VOLT ? op->volt_index[2] : op->curr_index[2])[n]);
            fld = fld + (VOLT ? op->volt_amp[n] : op->curr_amp[n]) * sig[exc_pos];
        }
    }
};

// AssignJobs2Threads (tools/useful.cpp:45-75)
std::vector<unsigned> assign_jobs(unsigned jobs, unsigned nthreads, bool remove_empty) {
    std::vector<unsigned> jpt;
    unsigned ui = jobs / nthreads;
    for (unsigned n = 0; n < nthreads; ++n) {
        jpt.push_back(ui);
        jobs -= ui;
    }
    for (unsigned n = 0; n < nthreads; ++n)
        if (jobs > 0) {
            ++jpt[n];
            --jobs;
        }
    if (remove_empty)
        while (!jpt.empty() && jpt.back() == 0) jpt.pop_back();
    return jpt;
}

// Runs iterTS steps of the multithreaded SSE-compressed engine.
void sse_mt_iterate(SSEEngine& S, BasicEngine& B, unsigned iterTS, unsigned nthreads) {
    std::vector<unsigned> jpt = assign_jobs(S.N[0], nthreads, true);
    nthreads = (unsigned)jpt.size();
    std::vector<unsigned> start(nthreads), stop(nthreads);
    start[0] = 0;
    stop[0] = jpt[0] - 1;
    for (unsigned n = 1; n < nthreads; ++n) {
        start[n] = stop[n - 1] + 1;
        stop[n] = start[n] + jpt[n] - 1;
    }
    // UPML per-thread x ranges (Engine_Ext_UPML::SetNumberOfThreads)
    const uint32_t nu = B.op->num_upml;
    std::vector<std::vector<unsigned>> u_num(nu), u_start(nu);
    for (uint32_t s = 0; s < nu; ++s) {
        u_num[s] = assign_jobs(B.op->upml[s].num_lines[0], nthreads, false);
        u_start[s].assign(nthreads, 0);
        for (unsigned n = 1; n < nthreads; ++n) u_start[s][n] = u_start[s][n - 1] + u_num[s][n - 1];
    }
    Barrier bar(nthreads);
    SSEHooks H{S, B};
    auto worker = [&](unsigned tid) {
        unsigned stop_h = (tid == nthreads - 1) ? stop[tid] - 1 : stop[tid];
        for (unsigned it = 0; it < iterTS; ++it) {
            unsigned ts = S.numTS + it;
            // DoPreVoltageUpdates: reverse priority order, barrier after each ext
            auto Vs = [&S](int n, uint32_t x, uint32_t y, uint32_t z) -> float& { return S.Vs(n, x, y, z); };
            if (tid == 0 && B.op->num_mur) B.mur(0, ts, Vs);
            bar.wait();
            if (tid == 0) H.ade_pre<true>();
            bar.wait();
            if (tid == 0) B.rlc_pre();
            bar.wait();
            for (uint32_t s = 0; s < nu; ++s) {
                H.upml<true, true>(s, u_start[s][tid], u_num[s][tid]);
                bar.wait();
            }
            S.update_voltages(start[tid], stop[tid] - start[tid] + 1);
            bar.wait();
            for (uint32_t s = nu; s-- > 0;) {
                H.upml<true, false>(s, u_start[s][tid], u_num[s][tid]);
                bar.wait();
            }
            if (tid == 0 && B.op->num_mur) B.mur(1, ts, Vs);
            bar.wait();
            if (tid == 0) B.rlc_apply(Vs);
            bar.wait();
            if (tid == 0) H.ade_apply<true>();
            bar.wait();
            if (tid == 0 && B.op->num_mur) B.mur(2, ts, Vs);
            bar.wait();
            if (tid == 0) H.excite<true>(ts);
            bar.wait();

            if (tid == 0) H.ade_pre<false>();
            bar.wait();
            for (uint32_t s = 0; s < nu; ++s) {
                H.upml<false, true>(s, u_start[s][tid], u_num[s][tid]);
                bar.wait();
            }
            S.update_currents(start[tid], stop_h - start[tid] + 1);
            bar.wait();
            for (uint32_t s = nu; s-- > 0;) {
                H.upml<false, false>(s, u_start[s][tid], u_num[s][tid]);
                bar.wait();
            }
            if (tid == 0) H.ade_apply<false>();
            bar.wait();
            if (tid == 0) H.excite<false>(ts);
            bar.wait();
        }
    };
    std::vector<std::thread> pool;
    for (unsigned t = 1; t < nthreads; ++t) pool.emplace_back(worker, t);
    worker(0);
    for (auto& th : pool) th.join();
    S.numTS += iterTS;
}

}  // namespace

extern "C" {

// Runs n_steps of the restated reference engine on desc.
//   engine: 0 = basic engine (Engine), 1 = SSE-compressed multithreaded
//   samples: rows of (2 + n_probes) doubles: ts, energy, probe values
//            (x weight); a row is recorded at every ts % interval == 0
//            (ts = 0 included) while ts <= n_steps; pass interval 0 for none.
//   returns the number of sample rows written (<= max_rows), or < 0.
//   final_volt / final_curr (may be NULL): [3][Nx][Ny][Nz] after the run.
//   seconds: wall time of the stepping only (probe sampling excluded).
long oracle_run(const fdtd_op_desc* desc, const fdtd_probe_desc* probes, int n_probes, unsigned n_steps,
                unsigned interval, int engine, int threads, int with_energy, double* samples, long max_rows,
                float* final_volt, float* final_curr, double* seconds) {
    if (!desc) return -1;
    BasicEngine B(desc);
    std::unique_ptr<SSEEngine> S;
    if (engine == 1) S.reset(new SSEEngine(desc));
    if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    int ncol = 0;  // sample columns: one per integral probe, three per field probe
    for (int p = 0; p < n_probes; ++p) ncol += (probes[p].type == 2 || probes[p].type == 3) ? 3 : 1;
    const int row = 2 + ncol;
    long rows = 0;
    double secs = 0;
    // field access for probes
    auto sync_to_basic = [&]() {
        if (!S) return;
        for (int n = 0; n < 3; ++n)
            for (uint32_t x = 0; x < B.N[0]; ++x)
                for (uint32_t y = 0; y < B.N[1]; ++y)
                    for (uint32_t z = 0; z < B.N[2]; ++z) {
                        B.V(n, x, y, z) = S->Vs(n, x, y, z);
                        B.I(n, x, y, z) = S->Is(n, x, y, z);
                    }
    };
    auto record = [&](unsigned ts) {
        if (!samples || rows >= max_rows) return;
        sync_to_basic();
        double* r = samples + rows * row;
        r[0] = ts;
        r[1] = with_energy ? B.fast_energy() : -1.0;
        int col = 2;
        for (int p = 0; p < n_probes; ++p) {
            const fdtd_probe_desc& pd = probes[p];
            if (pd.type == 2 || pd.type == 3) {  // ProcessFieldProbe: GetEField / GetHField, no interpolation
                for (int n = 0; n < 3; ++n) {
                    double v = 0;
                    if (pd.enabled) v = B.raw_field(pd.type == 3, n, pd.start);
                    r[col++] = v * pd.weight;
                }
                continue;
            }
            double v = 0;
            if (pd.enabled) v = (pd.type == 0) ? B.voltage_integral(pd.start, pd.stop) : B.current_integral(pd);
            r[col++] = v * pd.weight;
        }
        ++rows;
    };
    unsigned ts = 0;
    if (interval) record(0);
    while (ts < n_steps) {
        unsigned step = interval ? std::min(interval - ts % interval, n_steps - ts) : n_steps - ts;
        auto t0 = std::chrono::steady_clock::now();
        if (S) {
            sse_mt_iterate(*S, B, step, (unsigned)threads);
        } else {
            B.iterate(step);
        }
        secs += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        ts += step;
        if (interval && ts % interval == 0) record(ts);
    }
    if (S) sync_to_basic();
    size_t NN = (size_t)B.N[0] * B.N[1] * B.N[2];
    if (final_volt) std::memcpy(final_volt, B.volt.data(), 3 * NN * sizeof(float));
    if (final_curr) std::memcpy(final_curr, B.curr.data(), 3 * NN * sizeof(float));
    if (seconds) *seconds = secs;
    return rows;
}

}  // extern "C"
