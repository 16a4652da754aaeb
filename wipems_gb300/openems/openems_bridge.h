// openems_bridge.h -- builds the engine description of include/wipems_fdtd.h
// (fdtd_op_desc) from the arrays an openEMS Operator and its extensions hold
// after CalcECOperator.  It names no openEMS type: Operator_CUDA
// (operator_cuda.cpp) feeds it the operator's pointer trees, and a test can
// feed it trees of its own.
//
// openEMS stores an [n][x][y][z] array as a pointer tree made by
// Create_N_3DArray (tools/array_ops.h:113-147): a[n] -> a[n][x] -> a[n][x][y]
// -> one allocation per z-line.  The engine wants the same values
// contiguous, z fastest: base[((n*Nx + x)*Ny + y)*Nz + z].
#pragma once

#include <cstdint>
#include <cstring>
#include <memory>
#include <vector>

#include "../../include/wipems_fdtd.h"

namespace wipems_openems {

// [3][nx][ny][nz] pointer tree -> contiguous
template <class T>
void flatten_n3(T**** a, const uint32_t n[3], std::vector<float>& out) {
    out.resize(3 * (size_t)n[0] * n[1] * n[2]);
    float* o = out.data();
    for (int c = 0; c < 3; ++c)
        for (uint32_t x = 0; x < n[0]; ++x)
            for (uint32_t y = 0; y < n[1]; ++y) {
                const T* line = a[c][x][y];
                for (uint32_t z = 0; z < n[2]; ++z) *o++ = (float)line[z];
            }
}

// [n0][n1] pointer tree (Create2DArray, array_ops.h:71-85) -> contiguous
template <class T>
void flatten_2(T** a, uint32_t n0, uint32_t n1, std::vector<float>& out) {
    out.resize((size_t)n0 * n1);
    for (uint32_t i = 0; i < n0; ++i)
        for (uint32_t j = 0; j < n1; ++j) out[(size_t)i * n1 + j] = (float)a[i][j];
}

// [3][count] per-component lists -> contiguous (absent: empty)
template <class T>
void flatten_3xn(T** a, uint32_t count, std::vector<float>& out) {
    out.clear();
    if (!a) return;
    out.resize(3 * (size_t)count);
    for (int c = 0; c < 3; ++c)
        for (uint32_t i = 0; i < count; ++i) out[(size_t)c * count + i] = (float)a[c][i];
}

// The description and the host storage it points into.  Fill with the
// set_* / add_* calls, then finish(); desc stays valid while the view lives.
struct OperatorView {
    fdtd_op_desc desc{};
    std::vector<float> vv, vi, ii, iv;
    struct Slab {
        fdtd_upml_desc d{};
        std::vector<float> vv, vvfo, vvfn, ii, iifo, iifn;
    };
    std::vector<std::unique_ptr<Slab>> slabs;
    struct Ade {
        fdtd_ade_desc d{};
        std::vector<uint32_t> pos[3];
        std::vector<float> v_int, v_ext, v_lor, i_int, i_ext, i_lor;
    };
    std::vector<std::unique_ptr<Ade>> ade;
    std::vector<uint32_t> v_idx[3], c_idx[3], v_delay, c_delay;
    std::vector<uint16_t> v_dir, c_dir;
    std::vector<float> v_amp, c_amp, sig_v, sig_c;
    struct Mur {
        fdtd_mur_desc d{};
        std::vector<float> cp, cpp;
    };
    std::vector<std::unique_ptr<Mur>> mur;
    fdtd_rlc_desc rlc{};
    std::vector<uint32_t> rlc_pos[3];
    std::vector<int> rlc_dir;
    std::vector<float> rlc_c[9];  // ilv, i2v, vv2, vj1, vj2, vvd, ib0, b1, b2
    std::vector<double> lines[3];
    std::vector<fdtd_upml_desc> upml_arr;
    std::vector<fdtd_ade_desc> ade_arr;
    std::vector<fdtd_mur_desc> mur_arr;

    // Operator::vv / vi / ii / iv, numLines, dT, discLines, gridDelta
    template <class T>
    void set_main(T**** vv_, T**** vi_, T**** ii_, T**** iv_, const uint32_t n[3], double dT, double* const disc[3],
                  double unit) {
        for (int a = 0; a < 3; ++a) {
            desc.num_lines[a] = n[a];
            lines[a].assign(disc[a], disc[a] + n[a]);
        }
        desc.dT = dT;
        desc.unit = unit;
        flatten_n3(vv_, n, vv);
        flatten_n3(vi_, n, vi);
        flatten_n3(ii_, n, ii);
        flatten_n3(iv_, n, iv);
    }

    // one Operator_Ext_UPML (m_StartPos, m_numLines, vv ... iifn)
    template <class T>
    void add_upml(const uint32_t start[3], const uint32_t nl[3], T**** vv_, T**** vvfo_, T**** vvfn_, T**** ii_,
                  T**** iifo_, T**** iifn_) {
        std::unique_ptr<Slab> s(new Slab());
        for (int a = 0; a < 3; ++a) {
            s->d.start[a] = start[a];
            s->d.num_lines[a] = nl[a];
        }
        flatten_n3(vv_, nl, s->vv);
        flatten_n3(vvfo_, nl, s->vvfo);
        flatten_n3(vvfn_, nl, s->vvfn);
        flatten_n3(ii_, nl, s->ii);
        flatten_n3(iifo_, nl, s->iifo);
        flatten_n3(iifn_, nl, s->iifn);
        slabs.push_back(std::move(s));
    }

    // one dispersion order of Operator_Ext_LorentzMaterial: m_LM_Count[o],
    // m_LM_pos[o], the *_On flags and the [3][count] coefficient lists
    // (NULL where that part is off)
    template <class T>
    void add_ade_order(uint32_t count, unsigned int** pos, bool volt_on, bool curr_on, bool volt_lor_on,
                       bool curr_lor_on, T** v_int, T** v_ext, T** v_lor, T** i_int, T** i_ext, T** i_lor) {
        std::unique_ptr<Ade> a(new Ade());
        a->d.count = count;
        for (int n = 0; n < 3; ++n) a->pos[n].assign(pos[n], pos[n] + count);
        a->d.volt_on = volt_on;
        a->d.curr_on = curr_on;
        a->d.volt_lor_on = volt_lor_on;
        a->d.curr_lor_on = curr_lor_on;
        flatten_3xn(volt_on ? v_int : nullptr, count, a->v_int);
        flatten_3xn(volt_on ? v_ext : nullptr, count, a->v_ext);
        flatten_3xn(volt_lor_on ? v_lor : nullptr, count, a->v_lor);
        flatten_3xn(curr_on ? i_int : nullptr, count, a->i_int);
        flatten_3xn(curr_on ? i_ext : nullptr, count, a->i_ext);
        flatten_3xn(curr_lor_on ? i_lor : nullptr, count, a->i_lor);
        ade.push_back(std::move(a));
    }

    // Operator_Ext_Excitation's lists (one side: voltage or current)
    template <class T>
    void set_excitation(bool current, uint32_t count, unsigned int* const index[3], const unsigned short* dir,
                        const T* amp, const unsigned int* delay) {
        std::vector<uint32_t>* idx = current ? c_idx : v_idx;
        std::vector<uint16_t>& d = current ? c_dir : v_dir;
        std::vector<float>& a = current ? c_amp : v_amp;
        std::vector<uint32_t>& dl = current ? c_delay : v_delay;
        for (int n = 0; n < 3; ++n) idx[n].assign(index[n], index[n] + count);
        d.assign(dir, dir + count);
        a.assign(amp, amp + count);
        dl.assign(delay, delay + count);
    }

    // Excitation::GetVoltageSignal / GetCurrentSignal / GetLength
    template <class T>
    void set_signal(const T* volt, const T* curr, uint32_t length, uint32_t period_ts) {
        sig_v.assign(volt, volt + length);
        sig_c.assign(curr, curr + length);
        desc.signal_period_ts = period_ts;
    }

    // one Operator_Ext_Mur_ABC face
    template <class T>
    void add_mur(int ny, bool top, uint32_t line, uint32_t shift, uint32_t n_p, uint32_t n_pp, T** coef_p,
                 T** coef_pp, uint32_t start_ts) {
        std::unique_ptr<Mur> m(new Mur());
        m->d.ny = ny;
        m->d.top = top ? 1 : 0;
        m->d.line = line;
        m->d.shift = shift;
        m->d.n_p = n_p;
        m->d.n_pp = n_pp;
        m->d.start_ts = start_ts;
        flatten_2(coef_p, n_p, n_pp, m->cp);
        flatten_2(coef_pp, n_p, n_pp, m->cpp);
        mur.push_back(std::move(m));
    }

    // Operator_Ext_LumpedRLC's lists; coef = ilv, i2v, vv2, vj1, vj2, vvd, ib0, b1, b2
    template <class T>
    void set_rlc(uint32_t count, unsigned int* const pos[3], const int* dir, T* const coef[9]) {
        for (int n = 0; n < 3; ++n) rlc_pos[n].assign(pos[n], pos[n] + count);
        rlc_dir.assign(dir, dir + count);
        for (int k = 0; k < 9; ++k) rlc_c[k].assign(coef[k], coef[k] + count);
    }

    // points desc at the storage above
    void finish() {
        desc.vv = vv.data();
        desc.vi = vi.data();
        desc.ii = ii.data();
        desc.iv = iv.data();
        upml_arr.clear();
        for (const auto& s : slabs) {
            fdtd_upml_desc d = s->d;
            d.vv = s->vv.data();
            d.vvfo = s->vvfo.data();
            d.vvfn = s->vvfn.data();
            d.ii = s->ii.data();
            d.iifo = s->iifo.data();
            d.iifn = s->iifn.data();
            upml_arr.push_back(d);
        }
        desc.num_upml = (uint32_t)upml_arr.size();
        desc.upml = upml_arr.empty() ? nullptr : upml_arr.data();
        ade_arr.clear();
        for (const auto& a : ade) {
            fdtd_ade_desc d = a->d;
            for (int n = 0; n < 3; ++n) d.pos[n] = a->pos[n].data();
            d.v_int = a->v_int.empty() ? nullptr : a->v_int.data();
            d.v_ext = a->v_ext.empty() ? nullptr : a->v_ext.data();
            d.v_lor = a->v_lor.empty() ? nullptr : a->v_lor.data();
            d.i_int = a->i_int.empty() ? nullptr : a->i_int.data();
            d.i_ext = a->i_ext.empty() ? nullptr : a->i_ext.data();
            d.i_lor = a->i_lor.empty() ? nullptr : a->i_lor.data();
            ade_arr.push_back(d);
        }
        desc.num_ade_orders = (uint32_t)ade_arr.size();
        desc.ade = ade_arr.empty() ? nullptr : ade_arr.data();
        desc.volt_count = (uint32_t)v_amp.size();
        desc.curr_count = (uint32_t)c_amp.size();
        for (int n = 0; n < 3; ++n) {
            desc.volt_index[n] = v_idx[n].data();
            desc.curr_index[n] = c_idx[n].data();
            desc.lines[n] = lines[n].data();
        }
        desc.volt_dir = v_dir.data();
        desc.volt_amp = v_amp.data();
        desc.volt_delay = v_delay.data();
        desc.curr_dir = c_dir.data();
        desc.curr_amp = c_amp.data();
        desc.curr_delay = c_delay.data();
        desc.signal_length = (uint32_t)sig_v.size();
        desc.signal_volt = sig_v.data();
        desc.signal_curr = sig_c.data();
        mur_arr.clear();
        for (const auto& m : mur) {
            fdtd_mur_desc d = m->d;
            d.coef_p = m->cp.data();
            d.coef_pp = m->cpp.data();
            mur_arr.push_back(d);
        }
        desc.num_mur = (uint32_t)mur_arr.size();
        desc.mur = mur_arr.empty() ? nullptr : mur_arr.data();
        rlc.count = (uint32_t)rlc_dir.size();
        for (int n = 0; n < 3; ++n) rlc.pos[n] = rlc_pos[n].data();
        rlc.dir = rlc_dir.data();
        rlc.ilv = rlc_c[0].data();
        rlc.i2v = rlc_c[1].data();
        rlc.vv2 = rlc_c[2].data();
        rlc.vj1 = rlc_c[3].data();
        rlc.vj2 = rlc_c[4].data();
        rlc.vvd = rlc_c[5].data();
        rlc.ib0 = rlc_c[6].data();
        rlc.b1 = rlc_c[7].data();
        rlc.b2 = rlc_c[8].data();
        desc.rlc = rlc.count ? &rlc : nullptr;
    }
};

}  // namespace wipems_openems
