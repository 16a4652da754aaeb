// Test harness for wipems_gb300/openems/openems_bridge.h: rebuilds an engine
// description the way an openEMS operator holds it -- every array as a
// pointer tree with one allocation per z-line ([n][x][y] -> line), the
// dispersion lists as [3][count] pointer arrays, the Mur coefficients as
// [n_p] -> row arrays -- and runs it through the bridge (OperatorView), the
// code Operator_CUDA::Describe uses.  Loaded by the tests with ctypes.
#include <cstdint>
#include <cstring>
#include <memory>
#include <vector>

#include "../../wipems_gb300/openems/openems_bridge.h"

namespace {

struct Tree3 {  // float[3][nx][ny][nz] as a pointer tree, one block per z-line
    std::vector<std::unique_ptr<float[]>> blocks;
    std::vector<float*> lines;
    std::vector<float**> rows;
    std::vector<float***> comps;
    float**** root = nullptr;
    void make(const float* src, const uint32_t n[3]) {
        const size_t nn = (size_t)n[0] * n[1] * n[2];
        lines.resize(3 * (size_t)n[0] * n[1]);
        rows.resize(3 * (size_t)n[0]);
        comps.resize(3);
        for (int c = 0; c < 3; ++c) {
            for (uint32_t x = 0; x < n[0]; ++x) {
                for (uint32_t y = 0; y < n[1]; ++y) {
                    blocks.emplace_back(new float[n[2]]);
                    std::memcpy(blocks.back().get(), src + (size_t)c * nn + ((size_t)x * n[1] + y) * n[2],
                                n[2] * sizeof(float));
                    lines[((size_t)c * n[0] + x) * n[1] + y] = blocks.back().get();
                }
                rows[(size_t)c * n[0] + x] = &lines[((size_t)c * n[0] + x) * n[1]];
            }
            comps[c] = &rows[(size_t)c * n[0]];
        }
        root = comps.data();
    }
};

struct List3 {  // float[3][count] as three pointers
    std::vector<float> data;
    float* ptr[3] = {nullptr, nullptr, nullptr};
    float** get(const float* src, uint32_t count) {
        if (!src) return nullptr;
        data.assign(src, src + 3 * (size_t)count);
        for (int c = 0; c < 3; ++c) ptr[c] = &data[(size_t)c * count];
        return ptr;
    }
};

struct Harness {
    Tree3 main[4];
    std::vector<std::unique_ptr<Tree3>> upml;
    std::vector<std::unique_ptr<List3>> ade;
    std::vector<std::vector<unsigned int>> ade_pos;
    std::vector<unsigned int*> ade_pos_ptr;
    std::vector<std::vector<float>> mur_data;
    std::vector<std::vector<float*>> mur_rows;
    std::vector<unsigned int> rlc_pos_data[3];
    unsigned int* rlc_pos[3];
    std::vector<unsigned short> vdir, cdir;
    std::vector<unsigned int> vidx[3], cidx[3];
    unsigned int* vidx_p[3];
    unsigned int* cidx_p[3];
    double* lines[3];
    wipems_openems::OperatorView view;
};

}  // namespace

extern "C" {

void* bridge_build(const fdtd_op_desc* d) {
    std::unique_ptr<Harness> h(new Harness());
    const uint32_t* n = d->num_lines;
    const float* m[4] = {d->vv, d->vi, d->ii, d->iv};
    for (int k = 0; k < 4; ++k) h->main[k].make(m[k], n);
    for (int a = 0; a < 3; ++a) h->lines[a] = const_cast<double*>(d->lines[a]);
    h->view.set_main(h->main[0].root, h->main[1].root, h->main[2].root, h->main[3].root, n, d->dT, h->lines, d->unit);
    for (uint32_t s = 0; s < d->num_upml; ++s) {
        const fdtd_upml_desc& u = d->upml[s];
        const float* src[6] = {u.vv, u.vvfo, u.vvfn, u.ii, u.iifo, u.iifn};
        float**** t[6];
        for (int k = 0; k < 6; ++k) {
            h->upml.emplace_back(new Tree3());
            h->upml.back()->make(src[k], u.num_lines);
            t[k] = h->upml.back()->root;
        }
        h->view.add_upml(u.start, u.num_lines, t[0], t[1], t[2], t[3], t[4], t[5]);
    }
    h->ade_pos.resize(3 * (size_t)d->num_ade_orders);
    h->ade_pos_ptr.resize(3 * (size_t)d->num_ade_orders);
    for (uint32_t o = 0; o < d->num_ade_orders; ++o) {
        const fdtd_ade_desc& a = d->ade[o];
        for (int c = 0; c < 3; ++c) {
            h->ade_pos[3 * o + c].assign(a.pos[c], a.pos[c] + a.count);
            h->ade_pos_ptr[3 * o + c] = h->ade_pos[3 * o + c].data();
        }
        const float* src[6] = {a.v_int, a.v_ext, a.v_lor, a.i_int, a.i_ext, a.i_lor};
        float** l[6];
        for (int k = 0; k < 6; ++k) {
            h->ade.emplace_back(new List3());
            l[k] = h->ade.back()->get(src[k], a.count);
        }
        h->view.add_ade_order(a.count, &h->ade_pos_ptr[3 * o], a.volt_on != 0, a.curr_on != 0, a.volt_lor_on != 0,
                              a.curr_lor_on != 0, l[0], l[1], l[2], l[3], l[4], l[5]);
    }
    for (int c = 0; c < 3; ++c) {
        h->vidx[c].assign(d->volt_index[c], d->volt_index[c] + d->volt_count);
        h->cidx[c].assign(d->curr_index[c], d->curr_index[c] + d->curr_count);
        h->vidx_p[c] = h->vidx[c].data();
        h->cidx_p[c] = h->cidx[c].data();
    }
    h->vdir.assign(d->volt_dir, d->volt_dir + d->volt_count);
    h->cdir.assign(d->curr_dir, d->curr_dir + d->curr_count);
    h->view.set_excitation(false, d->volt_count, h->vidx_p, h->vdir.data(), d->volt_amp, d->volt_delay);
    h->view.set_excitation(true, d->curr_count, h->cidx_p, h->cdir.data(), d->curr_amp, d->curr_delay);
    h->view.set_signal(d->signal_volt, d->signal_curr, d->signal_length, d->signal_period_ts);
    for (uint32_t f = 0; f < d->num_mur; ++f) {
        const fdtd_mur_desc& M = d->mur[f];
        float** rows[2];
        for (int k = 0; k < 2; ++k) {
            const float* src = k ? M.coef_pp : M.coef_p;
            h->mur_data.emplace_back(src, src + (size_t)M.n_p * M.n_pp);
            h->mur_rows.emplace_back(M.n_p);
            for (uint32_t i = 0; i < M.n_p; ++i) h->mur_rows.back()[i] = &h->mur_data.back()[(size_t)i * M.n_pp];
            rows[k] = h->mur_rows.back().data();
        }
        h->view.add_mur(M.ny, M.top != 0, M.line, M.shift, M.n_p, M.n_pp, rows[0], rows[1], M.start_ts);
    }
    if (d->rlc && d->rlc->count) {
        const fdtd_rlc_desc& r = *d->rlc;
        for (int c = 0; c < 3; ++c) {
            h->rlc_pos_data[c].assign(r.pos[c], r.pos[c] + r.count);
            h->rlc_pos[c] = h->rlc_pos_data[c].data();
        }
        float* coef[9] = {const_cast<float*>(r.ilv), const_cast<float*>(r.i2v), const_cast<float*>(r.vv2),
                          const_cast<float*>(r.vj1), const_cast<float*>(r.vj2), const_cast<float*>(r.vvd),
                          const_cast<float*>(r.ib0), const_cast<float*>(r.b1),  const_cast<float*>(r.b2)};
        h->view.set_rlc(r.count, h->rlc_pos, r.dir, coef);
    }
    h->view.finish();
    return h.release();
}

const fdtd_op_desc* bridge_desc(void* h) { return &static_cast<Harness*>(h)->view.desc; }

void bridge_free(void* h) { delete static_cast<Harness*>(h); }

}  // extern "C"
