// Engine_CUDA: the device-resident FDTD time stepper behind the C ABI.
//
// fdtd_engine_create plays the part of Operator::CreateEngine + Engine::Init
// (FDTD/operator.cpp:63-67, FDTD/engine.cpp:49-57) for the CUDA engine: it
// compresses the reference-form coefficient arrays into one per-node tuple
// index (the Operator_SSE_Compressed idea, operator_sse_compressed.cpp:120-176,
// here per node and extended by the UPML / ADE / excitation terms the kernels
// fuse), uploads index + tables, and allocates the zeroed field arrays.
// fdtd_engine_iterate is Engine::IterateTS (engine.cpp:255-274): per
// timestep one voltage and one current kernel, with probe sampling and the
// energy reduction at the probe interval; chunks of one probe interval are
// captured once into a CUDA graph and replayed.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "fdtd_host.h"
#include "kernels.cuh"
#include "kernels_tma.cuh"

#include <cudaTypedefs.h>

namespace wipems {

namespace {

#define CK(call)                                                                   \
    do {                                                                           \
        cudaError_t e_ = (call);                                                   \
        if (e_ != cudaSuccess) {                                                   \
            set_error(std::string(#call) + ": " + cudaGetErrorString(e_));         \
            return FDTD_ERR_CUDA;                                                  \
        }                                                                          \
    } while (0)

// One compressed coefficient tuple: everything the two kernels read per node.
// Unused terms are zero so that equal tuples compare equal bytewise.
struct Tuple {
    float e[6];        // vv0..2, vi0..2
    float h[6];        // ii0..2, iv0..2
    uint32_t fe, fh;   // flags
    float eu[9];       // vvp, vvfo, vvfn
    float hu[9];       // iip, iifo, iifn
    float ea[9];       // v_int, v_ext, v_lor
    float ha[9];       // i_int, i_ext, i_lor
    float ex[3];       // volt excitation amplitude
    int32_t exd[3];    // volt excitation delay (-1 = none)
    float hx[3];
    int32_t hxd[3];
};

struct TupleHash {
    size_t operator()(const Tuple& t) const {
        const uint64_t* p = reinterpret_cast<const uint64_t*>(&t);
        uint64_t h = 1469598103934665603ull;
        for (size_t i = 0; i < sizeof(Tuple) / 8; ++i) {
            h ^= p[i] + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2);
        }
        return (size_t)h;
    }
};
struct TupleEq {
    bool operator()(const Tuple& a, const Tuple& b) const { return std::memcmp(&a, &b, sizeof(Tuple)) == 0; }
};
static_assert(sizeof(Tuple) % 8 == 0, "tuple must be 8-byte sized");

template <class T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
    int alloc(size_t count, uint64_t& total) {
        n = count;
        if (count == 0) return FDTD_OK;
        cudaError_t e = cudaMalloc(&p, count * sizeof(T));
        if (e != cudaSuccess) {
            p = nullptr;
            set_error(std::string("cudaMalloc: ") + cudaGetErrorString(e));
            return FDTD_ERR_NOMEM;
        }
        total += count * sizeof(T);
        return FDTD_OK;
    }
};

}  // namespace
}  // namespace wipems

using namespace wipems;

struct fdtd_engine_s {
    int device = 0;
    cudaStream_t stream = nullptr;
    uint32_t N[3];
    int Nzp = 0;
    long long comp = 0;
    double dT = 0;
    DevGrid g{};
    DevBuf<float> V, I, FV, FI, AV, LV, AI, LI;
    DevBuf<uint8_t> idx;
    DevBuf<float4> tabE, tabH, tabEU, tabHU, tabEA, tabHA, tabEX, tabHX;
    DevBuf<float> sigV, sigC;
    DevBuf<int> d_ts;
    DevBuf<double> d_eacc;
    DevBuf<double> d_energy_tmp;
    // probes
    std::vector<ProbeEntry> h_entries;
    std::vector<int> h_first{0};
    std::vector<double> h_weight;
    DevBuf<ProbeEntry> d_entries;
    DevBuf<int> d_first;
    DevBuf<double> d_weight;
    DevBuf<double> ring;
    DevBuf<int> d_nsamp;
    DevBuf<int> d_err;
    ProbeSet ps{};
    bool probes_uploaded = false;
    uint32_t interval = 0;
    bool energy_on_probe = true;
    bool use_graphs = true;
    uint32_t cap = 0;
    // state
    uint32_t ts = 0;
    bool started = false;
    bool need_initial_sample = true;
    int feat = 0;
    bool idx16 = true;
    int TY = 8;
    int XC = 16;
    bool use_tma = true;
    int stages = 3;
    int zw = 2;
    TmaMaps maps{};
    TileInfo ti{};
    size_t smem_bytes = 0;
    uint32_t num_tuples = 0, upml_nodes = 0, ade_nodes = 0;
    uint64_t device_bytes = 0;
    // graph of one probe interval
    cudaGraphExec_t chunk = nullptr;
    // timing
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    double last_ms = 0;
    uint64_t last_launches = 0;

    ~fdtd_engine_s() {
        if (chunk) cudaGraphExecDestroy(chunk);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace wipems {
namespace {

typedef void (*VoltFn)(DevGrid, int, int);
typedef void (*CurrFn)(DevGrid, int, int);

template <typename IdxT>
VoltFn pick_volt(int feat) {
    switch (feat) {
        case 0: return k_volt<IdxT, 0>;
        case 1: return k_volt<IdxT, 1>;
        case 2: return k_volt<IdxT, 2>;
        default: return k_volt<IdxT, 3>;
    }
}
template <typename IdxT>
CurrFn pick_curr(int feat, bool energy) {
    if (energy) {
        switch (feat) {
            case 0: return k_curr<IdxT, 0, true>;
            case 1: return k_curr<IdxT, 1, true>;
            case 2: return k_curr<IdxT, 2, true>;
            default: return k_curr<IdxT, 3, true>;
        }
    }
    switch (feat) {
        case 0: return k_curr<IdxT, 0, false>;
        case 1: return k_curr<IdxT, 1, false>;
        case 2: return k_curr<IdxT, 2, false>;
        default: return k_curr<IdxT, 3, false>;
    }
}

template <typename IdxT, int ZW>
void launch_tma_half_zw(fdtd_engine_s* e, int ts_off, bool energy, bool volt) {
    constexpr int TZ = 32 * ZW;
    dim3 block(32, TMA_TY);
    const bool up = (e->feat & FEAT_UPML) != 0;
    const int S = e->stages;
    const size_t sm = up ? StageLayout<IdxT, true, ZW>::smem(S) : StageLayout<IdxT, false, ZW>::smem(S);
    const DevGrid& g = e->g;
    const TmaMaps& m = e->maps;
    const TileInfo& ti = e->ti;
    const int XC = e->XC;
    if (volt) {
        dim3 gv((ti.ne[2] + TZ - 1) / TZ, (ti.ne[1] + TMA_TY - 1) / TMA_TY, (ti.ne[0] + XC - 1) / XC);
        switch (e->feat) {
            case 0: k_volt_tma<IdxT, 0, ZW><<<gv, block, sm, e->stream>>>(g, m, ti, ts_off, XC, S); break;
            case 1: k_volt_tma<IdxT, 1, ZW><<<gv, block, sm, e->stream>>>(g, m, ti, ts_off, XC, S); break;
            case 2: k_volt_tma<IdxT, 2, ZW><<<gv, block, sm, e->stream>>>(g, m, ti, ts_off, XC, S); break;
            default: k_volt_tma<IdxT, 3, ZW><<<gv, block, sm, e->stream>>>(g, m, ti, ts_off, XC, S); break;
        }
        return;
    }
    dim3 gc((e->N[2] - 1 + TZ - 1) / TZ, (e->N[1] - 1 + TMA_TY - 1) / TMA_TY, (e->N[0] - 1 + XC - 1) / XC);
    if (energy) {
        switch (e->feat) {
            case 0: k_curr_tma<IdxT, 0, true, ZW><<<gc, block, sm, e->stream>>>(g, m, ti, ts_off, XC, S); break;
            case 1: k_curr_tma<IdxT, 1, true, ZW><<<gc, block, sm, e->stream>>>(g, m, ti, ts_off, XC, S); break;
            case 2: k_curr_tma<IdxT, 2, true, ZW><<<gc, block, sm, e->stream>>>(g, m, ti, ts_off, XC, S); break;
            default: k_curr_tma<IdxT, 3, true, ZW><<<gc, block, sm, e->stream>>>(g, m, ti, ts_off, XC, S); break;
        }
    } else {
        switch (e->feat) {
            case 0: k_curr_tma<IdxT, 0, false, ZW><<<gc, block, sm, e->stream>>>(g, m, ti, ts_off, XC, S); break;
            case 1: k_curr_tma<IdxT, 1, false, ZW><<<gc, block, sm, e->stream>>>(g, m, ti, ts_off, XC, S); break;
            case 2: k_curr_tma<IdxT, 2, false, ZW><<<gc, block, sm, e->stream>>>(g, m, ti, ts_off, XC, S); break;
            default: k_curr_tma<IdxT, 3, false, ZW><<<gc, block, sm, e->stream>>>(g, m, ti, ts_off, XC, S); break;
        }
    }
}

template <typename IdxT>
void launch_tma_half(fdtd_engine_s* e, int ts_off, bool energy, bool volt) {
    if (e->zw == 2)
        launch_tma_half_zw<IdxT, 2>(e, ts_off, energy, volt);
    else
        launch_tma_half_zw<IdxT, 1>(e, ts_off, energy, volt);
}

template <typename IdxT>
void launch_tma(fdtd_engine_s* e, int ts_off, bool energy) {
    launch_tma_half<IdxT>(e, ts_off, energy, true);
    launch_tma_half<IdxT>(e, ts_off, energy, false);
}

int launch_step(fdtd_engine_s* e, int ts_off, bool energy) {
    if (e->use_tma) {
        if (e->idx16)
            launch_tma<uint16_t>(e, ts_off, energy);
        else
            launch_tma<uint32_t>(e, ts_off, energy);
        e->last_launches += 2;
        cudaError_t err = cudaGetLastError();
        if (err != cudaSuccess) {
            set_error(std::string("kernel launch: ") + cudaGetErrorString(err));
            return FDTD_ERR_CUDA;
        }
        return FDTD_OK;
    }
    dim3 block(32, e->TY);
    dim3 gv((e->N[2] + 31) / 32, (e->N[1] + e->TY - 1) / e->TY, (e->N[0] + e->XC - 1) / e->XC);
    dim3 gc((e->N[2] + 31) / 32, (e->N[1] + e->TY - 1) / e->TY, (e->N[0] - 1 + e->XC - 1) / e->XC);
    VoltFn fv = e->idx16 ? pick_volt<uint16_t>(e->feat) : pick_volt<uint32_t>(e->feat);
    CurrFn fc = e->idx16 ? pick_curr<uint16_t>(e->feat, energy) : pick_curr<uint32_t>(e->feat, energy);
    fv<<<gv, block, e->smem_bytes, e->stream>>>(e->g, ts_off, e->XC);
    fc<<<gc, block, e->smem_bytes, e->stream>>>(e->g, ts_off, e->XC);
    e->last_launches += 2;
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) {
        set_error(std::string("kernel launch: ") + cudaGetErrorString(err));
        return FDTD_ERR_CUDA;
    }
    return FDTD_OK;
}

int launch_advance(fdtd_engine_s* e, int adv, bool sample, bool energy_valid) {
    k_advance_sample<<<1, 256, 0, e->stream>>>(e->d_ts.p, adv, sample ? 1 : 0, e->ps, e->g,
                                                energy_valid ? 1 : 0, kEps0, kMue0);
    e->last_launches += 1;
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) {
        set_error(std::string("kernel launch: ") + cudaGetErrorString(err));
        return FDTD_ERR_CUDA;
    }
    return FDTD_OK;
}

int upload_probes(fdtd_engine_s* e) {
    if (e->probes_uploaded) return FDTD_OK;
    uint32_t np = (uint32_t)e->h_weight.size();
    int rc;
    if ((rc = e->d_entries.alloc(std::max<size_t>(1, e->h_entries.size()), e->device_bytes))) return rc;
    if ((rc = e->d_first.alloc(np + 1, e->device_bytes))) return rc;
    if ((rc = e->d_weight.alloc(std::max<uint32_t>(1, np), e->device_bytes))) return rc;
    if (!e->h_entries.empty())
        CK(cudaMemcpyAsync(e->d_entries.p, e->h_entries.data(), e->h_entries.size() * sizeof(ProbeEntry),
                           cudaMemcpyHostToDevice, e->stream));
    CK(cudaMemcpyAsync(e->d_first.p, e->h_first.data(), (np + 1) * sizeof(int), cudaMemcpyHostToDevice, e->stream));
    if (np)
        CK(cudaMemcpyAsync(e->d_weight.p, e->h_weight.data(), np * sizeof(double), cudaMemcpyHostToDevice,
                           e->stream));
    int row = 2 + (int)np;
    if ((rc = e->ring.alloc((size_t)e->cap * row, e->device_bytes))) return rc;
    e->ps.entries = e->d_entries.p;
    e->ps.first = e->d_first.p;
    e->ps.weight = e->d_weight.p;
    e->ps.nprobe = (int)np;
    e->ps.row_doubles = row;
    e->ps.ring = e->ring.p;
    e->ps.cap = (int)e->cap;
    e->ps.d_nsamp = e->d_nsamp.p;
    e->ps.d_err = e->d_err.p;
    e->probes_uploaded = true;
    return FDTD_OK;
}

int build_chunk_graph(fdtd_engine_s* e) {
    if (e->chunk) return FDTD_OK;
    cudaGraph_t graph = nullptr;
    CK(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
    int rc = FDTD_OK;
    uint64_t saved = e->last_launches;
    for (uint32_t k = 0; k < e->interval && rc == FDTD_OK; ++k)
        rc = launch_step(e, (int)k, e->energy_on_probe && (k + 1 == e->interval));
    if (rc == FDTD_OK) rc = launch_advance(e, (int)e->interval, true, e->energy_on_probe);
    e->last_launches = saved;
    cudaError_t ce = cudaStreamEndCapture(e->stream, &graph);
    if (rc != FDTD_OK) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    if (ce != cudaSuccess) {
        set_error(std::string("cudaStreamEndCapture: ") + cudaGetErrorString(ce));
        return FDTD_ERR_CUDA;
    }
    ce = cudaGraphInstantiate(&e->chunk, graph, 0);
    cudaGraphDestroy(graph);
    if (ce != cudaSuccess) {
        e->chunk = nullptr;
        set_error(std::string("cudaGraphInstantiate: ") + cudaGetErrorString(ce));
        return FDTD_ERR_CUDA;
    }
    return FDTD_OK;
}

// -------------------------------------------------------------- compression
struct NodeMaps {
    std::vector<int8_t> slab;           // UPML slab id per node or -1
    std::vector<int32_t> ade;           // ADE list position (order 0) or -1
    std::unordered_map<uint64_t, uint32_t> vexc, cexc;  // node*3+dir -> list entry
};

int compress(const fdtd_op_desc* d, fdtd_engine_s* e, std::vector<uint32_t>& node_idx, std::vector<Tuple>& tuples,
             int threads) {
    const uint32_t Nx = d->num_lines[0], Ny = d->num_lines[1], Nz = d->num_lines[2];
    const size_t NN = (size_t)Nx * Ny * Nz;
    NodeMaps m;
    if (d->num_upml) {
        m.slab.assign(NN, -1);
        for (uint32_t s = 0; s < d->num_upml; ++s) {
            const fdtd_upml_desc& u = d->upml[s];
            for (uint32_t a = 0; a < 3; ++a)
                if (u.start[a] + u.num_lines[a] > d->num_lines[a]) {
                    set_error("UPML slab exceeds the grid");
                    return FDTD_ERR_ARG;
                }
            for (uint32_t x = 0; x < u.num_lines[0]; ++x)
                for (uint32_t y = 0; y < u.num_lines[1]; ++y)
                    for (uint32_t z = 0; z < u.num_lines[2]; ++z) {
                        size_t gi = ((size_t)(x + u.start[0]) * Ny + (y + u.start[1])) * Nz + (z + u.start[2]);
                        if (m.slab[gi] >= 0) {
                            set_error("UPML slabs overlap");
                            return FDTD_ERR_ARG;
                        }
                        m.slab[gi] = (int8_t)s;
                    }
        }
    }
    if (d->num_ade_orders > 1) {
        set_error("dispersion order > 1 is not provided by the fused kernels");
        return FDTD_ERR_UNSUPPORTED;
    }
    const fdtd_ade_desc* A = d->num_ade_orders ? &d->ade[0] : nullptr;
    if (A && A->curr_on) {
        // magnetic dispersion: supported by the kernels through the H tables
    }
    if (A) {
        m.ade.assign(NN, -1);
        for (uint32_t i = 0; i < A->count; ++i) {
            uint32_t x = A->pos[0][i], y = A->pos[1][i], z = A->pos[2][i];
            if (x >= Nx || y >= Ny || z >= Nz) {
                set_error("ADE position outside the grid");
                return FDTD_ERR_ARG;
            }
            m.ade[((size_t)x * Ny + y) * Nz + z] = (int32_t)i;
        }
    }
    for (uint32_t i = 0; i < d->volt_count; ++i) {
        uint32_t x = d->volt_index[0][i], y = d->volt_index[1][i], z = d->volt_index[2][i];
        if (x >= Nx || y >= Ny || z >= Nz || d->volt_dir[i] > 2) {
            set_error("voltage excitation outside the grid");
            return FDTD_ERR_ARG;
        }
        uint64_t key = (((uint64_t)x * Ny + y) * Nz + z) * 3 + d->volt_dir[i];
        if (m.vexc.count(key)) {
            set_error("duplicate voltage excitation on one edge");
            return FDTD_ERR_ARG;
        }
        m.vexc[key] = i;
    }
    for (uint32_t i = 0; i < d->curr_count; ++i) {
        uint32_t x = d->curr_index[0][i], y = d->curr_index[1][i], z = d->curr_index[2][i];
        if (x >= Nx - 1 || y >= Ny - 1 || z >= Nz - 1 || d->curr_dir[i] > 2) {
            set_error("current excitation outside the current domain");
            return FDTD_ERR_ARG;
        }
        uint64_t key = (((uint64_t)x * Ny + y) * Nz + z) * 3 + d->curr_dir[i];
        if (m.cexc.count(key)) {
            set_error("duplicate current excitation on one edge");
            return FDTD_ERR_ARG;
        }
        m.cexc[key] = i;
    }

    node_idx.assign(NN, 0);
    // Build tuples per x-plane in parallel, dedup per plane, then merge.
    std::vector<std::vector<Tuple>> plane_tuples(Nx);
    std::vector<std::vector<uint32_t>> plane_local(Nx);
    uint32_t upml_nodes = 0, ade_nodes = 0;
    std::vector<uint32_t> cnt_u(Nx, 0), cnt_a(Nx, 0);
    auto worker = [&](uint32_t x) {
        std::unordered_map<Tuple, uint32_t, TupleHash, TupleEq> local;
        std::vector<Tuple>& pt = plane_tuples[x];
        std::vector<uint32_t>& pl = plane_local[x];
        pl.resize((size_t)Ny * Nz);
        Tuple last;
        uint32_t last_id = UINT32_MAX;
        for (uint32_t y = 0; y < Ny; ++y)
            for (uint32_t z = 0; z < Nz; ++z) {
                const size_t gi = ((size_t)x * Ny + y) * Nz + z;
                Tuple t;
                std::memset(&t, 0, sizeof(t));
                for (int n = 0; n < 3; ++n) {
                    t.e[n] = d->vv[n * NN + gi];
                    t.e[3 + n] = d->vi[n * NN + gi];
                    t.h[n] = d->ii[n * NN + gi];
                    t.h[3 + n] = d->iv[n * NN + gi];
                    t.exd[n] = -1;
                    t.hxd[n] = -1;
                }
                if (!m.slab.empty() && m.slab[gi] >= 0) {
                    const fdtd_upml_desc& u = d->upml[m.slab[gi]];
                    size_t nloc = (size_t)u.num_lines[0] * u.num_lines[1] * u.num_lines[2];
                    size_t li = ((size_t)(x - u.start[0]) * u.num_lines[1] + (y - u.start[1])) * u.num_lines[2] +
                                (z - u.start[2]);
                    for (int n = 0; n < 3; ++n) {
                        t.eu[n] = u.vv[n * nloc + li];
                        t.eu[3 + n] = u.vvfo[n * nloc + li];
                        t.eu[6 + n] = u.vvfn[n * nloc + li];
                        t.hu[n] = u.ii[n * nloc + li];
                        t.hu[3 + n] = u.iifo[n * nloc + li];
                        t.hu[6 + n] = u.iifn[n * nloc + li];
                    }
                    t.fe |= TF_UPML;
                    t.fh |= TF_UPML;
                    cnt_u[x]++;
                }
                if (A && m.ade[gi] >= 0) {
                    uint32_t i = (uint32_t)m.ade[gi];
                    if (A->volt_on) {
                        bool lor = false;
                        for (int n = 0; n < 3; ++n) {
                            t.ea[n] = A->v_int[n * A->count + i];
                            t.ea[3 + n] = A->v_ext[n * A->count + i];
                            t.ea[6 + n] = (A->volt_lor_on && A->v_lor) ? A->v_lor[n * A->count + i] : 0.f;
                            if (t.ea[6 + n] != 0.f) lor = true;
                        }
                        t.fe |= TF_ADE | (lor ? TF_LOR : 0u);
                    }
                    if (A->curr_on) {
                        bool lor = false;
                        for (int n = 0; n < 3; ++n) {
                            t.ha[n] = A->i_int[n * A->count + i];
                            t.ha[3 + n] = A->i_ext[n * A->count + i];
                            t.ha[6 + n] = (A->curr_lor_on && A->i_lor) ? A->i_lor[n * A->count + i] : 0.f;
                            if (t.ha[6 + n] != 0.f) lor = true;
                        }
                        t.fh |= TF_ADE | (lor ? TF_LOR : 0u);
                    }
                    cnt_a[x]++;
                }
                if (!m.vexc.empty())
                    for (int n = 0; n < 3; ++n) {
                        auto it = m.vexc.find((uint64_t)gi * 3 + n);
                        if (it != m.vexc.end()) {
                            t.ex[n] = d->volt_amp[it->second];
                            t.exd[n] = (int32_t)d->volt_delay[it->second];
                            t.fe |= TF_EXC;
                        }
                    }
                if (!m.cexc.empty())
                    for (int n = 0; n < 3; ++n) {
                        auto it = m.cexc.find((uint64_t)gi * 3 + n);
                        if (it != m.cexc.end()) {
                            t.hx[n] = d->curr_amp[it->second];
                            t.hxd[n] = (int32_t)d->curr_delay[it->second];
                            t.fh |= TF_EXC;
                        }
                    }
                uint32_t id;
                if (last_id != UINT32_MAX && std::memcmp(&t, &last, sizeof(Tuple)) == 0) {
                    id = last_id;
                } else {
                    auto it = local.find(t);
                    if (it == local.end()) {
                        id = (uint32_t)pt.size();
                        local.emplace(t, id);
                        pt.push_back(t);
                    } else {
                        id = it->second;
                    }
                    last = t;
                    last_id = id;
                }
                pl[(size_t)y * Nz + z] = id;
            }
    };
    {
        std::atomic<uint32_t> next{0};
        std::vector<std::thread> pool;
        int nt = std::max(1, std::min<int>(threads, (int)Nx));
        for (int t = 0; t < nt; ++t)
            pool.emplace_back([&] {
                for (;;) {
                    uint32_t x = next.fetch_add(1);
                    if (x >= Nx) break;
                    worker(x);
                }
            });
        for (auto& th : pool) th.join();
    }
    std::unordered_map<Tuple, uint32_t, TupleHash, TupleEq> global;
    tuples.clear();
    for (uint32_t x = 0; x < Nx; ++x) {
        std::vector<uint32_t> remap(plane_tuples[x].size());
        for (size_t k = 0; k < plane_tuples[x].size(); ++k) {
            auto it = global.find(plane_tuples[x][k]);
            if (it == global.end()) {
                uint32_t id = (uint32_t)tuples.size();
                global.emplace(plane_tuples[x][k], id);
                tuples.push_back(plane_tuples[x][k]);
                remap[k] = id;
            } else {
                remap[k] = it->second;
            }
        }
        const std::vector<uint32_t>& pl = plane_local[x];
        for (size_t k = 0; k < pl.size(); ++k) node_idx[(size_t)x * Ny * Nz + k] = remap[pl[k]];
        upml_nodes += cnt_u[x];
        ade_nodes += cnt_a[x];
        std::vector<Tuple>().swap(plane_tuples[x]);
        std::vector<uint32_t>().swap(plane_local[x]);
    }
    e->upml_nodes = upml_nodes;
    e->ade_nodes = ade_nodes;
    return FDTD_OK;
}

void pack4(std::vector<float4>& out, size_t entry, int per, const float* vals, int nvals) {
    float* f = reinterpret_cast<float*>(&out[entry * per]);
    for (int k = 0; k < nvals; ++k) f[k] = vals[k];
}

}  // namespace
}  // namespace wipems

// Host-side compressed operator: per-node tuple index (padded device layout)
// plus the coefficient tables, ready to be copied to the device.
struct fdtd_cop_s {
    uint32_t N[3] = {0, 0, 0};
    int Nzp = 0;
    long long comp = 0;
    bool idx16 = true;
    uint8_t* idx = nullptr;  // pinned when a CUDA device is present
    bool idx_pinned = false;
    size_t idx_bytes = 0;
    std::vector<float4> hE, hH, hEU, hHU, hEA, hHA, hEX, hHX;
    std::vector<float> sigV, sigC;
    uint32_t sig_len = 0, sig_period = 0;
    int feat = 0;
    bool any_upml = false, any_ade_e = false, any_ade_h = false, any_lor_e = false, any_lor_h = false;
    uint32_t num_tuples = 0, upml_nodes = 0, ade_nodes = 0;
    int inner_lo[3] = {0, 0, 0}, inner_hi[3] = {0, 0, 0};  // nodes outside are (possibly) UPML
    bool trim_e[3] = {false, false, false};  // last line of the axis is inert for the voltage update
    double dT = 0;
    ~fdtd_cop_s() {
        if (idx) {
            if (idx_pinned)
                cudaFreeHost(idx);
            else
                std::free(idx);
        }
    }
};

namespace wipems {
namespace {

int compress_op(const fdtd_op_desc* d, fdtd_cop_s* c) {
    for (int a = 0; a < 3; ++a) {
        if (d->num_lines[a] < 2) {
            set_error("every axis needs at least two lines");
            return FDTD_ERR_ARG;
        }
        c->N[a] = d->num_lines[a];
    }
    if (!d->vv || !d->vi || !d->ii || !d->iv) {
        set_error("coefficient arrays missing");
        return FDTD_ERR_ARG;
    }
    if ((d->volt_count || d->curr_count) && (!d->signal_length || !d->signal_volt || !d->signal_curr)) {
        set_error("excitation points without an excitation signal");
        return FDTD_ERR_ARG;
    }
    c->dT = d->dT;
    fdtd_engine_s dummy;  // receives node counts
    std::vector<uint32_t> node_idx;
    std::vector<Tuple> tuples;
    int threads = (int)std::max(1u, std::thread::hardware_concurrency());
    int rc = compress(d, &dummy, node_idx, tuples, threads);
    if (rc) return rc;
    c->upml_nodes = dummy.upml_nodes;
    c->ade_nodes = dummy.ade_nodes;
    c->num_tuples = (uint32_t)tuples.size();
    c->idx16 = tuples.size() <= 65536;
    const uint32_t Nx = c->N[0], Ny = c->N[1], Nz = c->N[2];
    c->Nzp = (int)((Nz + 31) / 32 * 32);
    c->comp = (long long)Nx * Ny * c->Nzp;
    for (const Tuple& t : tuples) {
        c->any_upml |= (t.fe & TF_UPML) != 0;
        c->any_ade_e |= (t.fe & TF_ADE) != 0;
        c->any_ade_h |= (t.fh & TF_ADE) != 0;
        c->any_lor_e |= (t.fe & TF_LOR) != 0;
        c->any_lor_h |= (t.fh & TF_LOR) != 0;
    }
    c->feat = (c->any_upml ? FEAT_UPML : 0) | ((c->any_ade_e || c->any_ade_h) ? FEAT_ADE : 0);
    const size_t T = tuples.size();
    const float4 z4 = make_float4(0, 0, 0, 0);
    c->hE.assign(2 * T, z4);
    c->hH.assign(2 * T, z4);
    c->hEX.assign(2 * T, z4);
    c->hHX.assign(2 * T, z4);
    if (c->any_upml) {
        c->hEU.assign(3 * T, z4);
        c->hHU.assign(3 * T, z4);
    }
    if (c->feat & FEAT_ADE) {
        c->hEA.assign(3 * T, z4);
        c->hHA.assign(3 * T, z4);
    }
    for (size_t k = 0; k < T; ++k) {
        const Tuple& t = tuples[k];
        float e8[8] = {t.e[0], t.e[1], t.e[2], t.e[3], t.e[4], t.e[5], 0, 0};
        std::memcpy(&e8[6], &t.fe, 4);
        pack4(c->hE, k, 2, e8, 8);
        float h8[8] = {t.h[0], t.h[1], t.h[2], t.h[3], t.h[4], t.h[5], 0, 0};
        std::memcpy(&h8[6], &t.fh, 4);
        pack4(c->hH, k, 2, h8, 8);
        if (c->any_upml) {
            pack4(c->hEU, k, 3, t.eu, 9);
            pack4(c->hHU, k, 3, t.hu, 9);
        }
        if (c->feat & FEAT_ADE) {
            pack4(c->hEA, k, 3, t.ea, 9);
            pack4(c->hHA, k, 3, t.ha, 9);
        }
        float x8[8] = {t.ex[0], t.ex[1], t.ex[2], 0, 0, 0, 0, 0};
        std::memcpy(&x8[4], t.exd, 12);
        pack4(c->hEX, k, 2, x8, 8);
        float y8[8] = {t.hx[0], t.hx[1], t.hx[2], 0, 0, 0, 0, 0};
        std::memcpy(&y8[4], t.hxd, 12);
        pack4(c->hHX, k, 2, y8, 8);
    }
    const size_t ib = c->idx16 ? 2 : 4;
    c->idx_bytes = (size_t)c->comp * ib;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) == cudaSuccess && ndev > 0 &&
        cudaMallocHost(reinterpret_cast<void**>(&c->idx), c->idx_bytes) == cudaSuccess) {
        c->idx_pinned = true;
    } else {
        cudaGetLastError();  // clear the sticky "no device" error of the probe
        c->idx = static_cast<uint8_t*>(std::malloc(c->idx_bytes));
        if (!c->idx) {
            set_error("host allocation of the tuple index failed");
            return FDTD_ERR_NOMEM;
        }
    }
    std::memset(c->idx, 0, c->idx_bytes);
    for (uint32_t x = 0; x < Nx; ++x)
        for (uint32_t y = 0; y < Ny; ++y) {
            const size_t src = ((size_t)x * Ny + y) * Nz;
            const size_t dst = ((size_t)x * Ny + y) * c->Nzp;
            if (c->idx16) {
                uint16_t* p = reinterpret_cast<uint16_t*>(c->idx) + dst;
                for (uint32_t z = 0; z < Nz; ++z) p[z] = (uint16_t)node_idx[src + z];
            } else {
                uint32_t* p = reinterpret_cast<uint32_t*>(c->idx) + dst;
                for (uint32_t z = 0; z < Nz; ++z) p[z] = node_idx[src + z];
            }
        }
    // An axis' last line is inert for the voltage update when every node on it
    // has only PEC voltage edges (vv = vi = 0), no ADE / excitation and, in
    // UPML slabs, vvp = vvfo = 0: starting from zero its voltages stay zero.
    {
        std::vector<uint8_t> inert(tuples.size());
        for (size_t k = 0; k < tuples.size(); ++k) {
            const Tuple& t = tuples[k];
            bool z = true;
            for (int n = 0; n < 6; ++n) z = z && t.e[n] == 0.f;
            if (t.fe & (TF_ADE | TF_EXC)) z = false;
            if (t.fe & TF_UPML)
                for (int n = 0; n < 6; ++n) z = z && t.eu[n] == 0.f;
            inert[k] = z;
        }
        for (int a = 0; a < 3; ++a) {
            bool all = true;
            uint32_t pos[3];
            const int b = (a + 1) % 3, cc = (a + 2) % 3;
            pos[a] = c->N[a] - 1;
            for (pos[b] = 0; pos[b] < c->N[b] && all; ++pos[b])
                for (pos[cc] = 0; pos[cc] < c->N[cc] && all; ++pos[cc]) {
                    const size_t gi = ((size_t)pos[0] * Ny + pos[1]) * Nz + pos[2];
                    all = inert[node_idx[gi]] != 0;
                }
            c->trim_e[a] = all;
        }
    }
    // inner box outside of which UPML slabs lie (slabs touching a face)
    for (int a = 0; a < 3; ++a) {
        c->inner_lo[a] = 0;
        c->inner_hi[a] = (int)c->N[a] - 1;
    }
    for (uint32_t k = 0; k < d->num_upml; ++k) {
        const fdtd_upml_desc& u = d->upml[k];
        for (int a = 0; a < 3; ++a) {
            if (u.num_lines[a] == c->N[a]) continue;
            if (u.start[a] == 0) c->inner_lo[a] = std::max(c->inner_lo[a], (int)u.num_lines[a]);
            if (u.start[a] + u.num_lines[a] == c->N[a]) c->inner_hi[a] = std::min(c->inner_hi[a], (int)u.start[a] - 1);
        }
    }
    c->sig_len = d->signal_length;
    c->sig_period = d->signal_period_ts;
    if (d->signal_length) {
        c->sigV.assign(d->signal_volt, d->signal_volt + d->signal_length);
        c->sigC.assign(d->signal_curr, d->signal_curr + d->signal_length);
    }
    return FDTD_OK;
}

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

// 4-D map over one field array [3][Nx][Ny][Nzp] (dims z, y, x, component)
int field_map(CUtensorMap* m, float* base, const fdtd_engine_s* e, uint32_t box_z, uint32_t box_y) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc) {
        set_error("cuTensorMapEncodeTiled is not available from the driver");
        return FDTD_ERR_CUDA;
    }
    cuuint64_t dims[4] = {e->N[2], e->N[1], e->N[0], 3};
    cuuint64_t strides[3] = {(cuuint64_t)e->Nzp * 4, (cuuint64_t)e->N[1] * e->Nzp * 4, (cuuint64_t)e->comp * 4};
    cuuint32_t box[4] = {box_z, box_y, 1, 3};
    cuuint32_t es[4] = {1, 1, 1, 1};
    CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                     CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled (field) failed: " + std::to_string((int)r));
        return FDTD_ERR_CUDA;
    }
    return FDTD_OK;
}

int index_map(CUtensorMap* m, void* base, const fdtd_engine_s* e, uint32_t box_z) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc) {
        set_error("cuTensorMapEncodeTiled is not available from the driver");
        return FDTD_ERR_CUDA;
    }
    const cuuint64_t ib = e->idx16 ? 2 : 4;
    cuuint64_t dims[3] = {e->N[2], e->N[1], e->N[0]};
    cuuint64_t strides[2] = {(cuuint64_t)e->Nzp * ib, (cuuint64_t)e->N[1] * e->Nzp * ib};
    cuuint32_t box[3] = {box_z, TMA_TY, 1};
    cuuint32_t es[3] = {1, 1, 1};
    CUresult r = enc(m, e->idx16 ? CU_TENSOR_MAP_DATA_TYPE_UINT16 : CU_TENSOR_MAP_DATA_TYPE_UINT32, 3, base, dims,
                     strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled (index) failed: " + std::to_string((int)r));
        return FDTD_ERR_CUDA;
    }
    return FDTD_OK;
}

int make_maps(fdtd_engine_s* e) {
    int rc;
    const uint32_t TZ = 32u * (uint32_t)e->zw;
    if ((rc = field_map(&e->maps.I_halo, e->I.p, e, TZ + 4, TMA_TY + 1)) ||
        (rc = field_map(&e->maps.I_own, e->I.p, e, TZ, TMA_TY)) ||
        (rc = field_map(&e->maps.V_halo, e->V.p, e, TZ + 4, TMA_TY + 1)) ||
        (rc = field_map(&e->maps.V_own, e->V.p, e, TZ, TMA_TY)) || (rc = index_map(&e->maps.idx, e->idx.p, e, TZ)))
        return rc;
    if (e->FV.p && ((rc = field_map(&e->maps.FV_own, e->FV.p, e, TZ, TMA_TY)) ||
                    (rc = field_map(&e->maps.FI_own, e->FI.p, e, TZ, TMA_TY))))
        return rc;
    return FDTD_OK;
}

template <typename IdxT, int FEAT, int ZW>
cudaError_t set_attr_one(int bytes) {
    cudaError_t e1 = cudaFuncSetAttribute(k_volt_tma<IdxT, FEAT, ZW>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaError_t e2 = cudaFuncSetAttribute(k_curr_tma<IdxT, FEAT, true, ZW>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaError_t e3 = cudaFuncSetAttribute(k_curr_tma<IdxT, FEAT, false, ZW>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    return e1 != cudaSuccess ? e1 : (e2 != cudaSuccess ? e2 : e3);
}

int set_smem_attrs(int bytes) {
    cudaError_t r = cudaSuccess;
    cudaError_t t;
#define WIPEMS_ATTR(I, F)                                                  \
    if ((t = set_attr_one<I, F, 1>(bytes)) != cudaSuccess) r = t;          \
    if ((t = set_attr_one<I, F, 2>(bytes)) != cudaSuccess) r = t;
    WIPEMS_ATTR(uint16_t, 0) WIPEMS_ATTR(uint16_t, 1) WIPEMS_ATTR(uint16_t, 2) WIPEMS_ATTR(uint16_t, 3)
    WIPEMS_ATTR(uint32_t, 0) WIPEMS_ATTR(uint32_t, 1) WIPEMS_ATTR(uint32_t, 2) WIPEMS_ATTR(uint32_t, 3)
#undef WIPEMS_ATTR
    if (r != cudaSuccess) {
        set_error(std::string("cudaFuncSetAttribute(MaxDynamicSharedMemorySize): ") + cudaGetErrorString(r));
        return FDTD_ERR_CUDA;
    }
    return FDTD_OK;
}

// Engine::Init state: all fields and extension states zero, numTS = 0,
// no recorded samples (the ts = 0 sample is taken again on the next iterate).
int reset_state(fdtd_engine_s* e) {
    cudaStream_t s = e->stream;
    const size_t F = 3 * (size_t)e->comp * sizeof(float);
    for (DevBuf<float>* b : {&e->V, &e->I, &e->FV, &e->FI, &e->AV, &e->LV, &e->AI, &e->LI})
        if (b->p) CK(cudaMemsetAsync(b->p, 0, F, s));
    CK(cudaMemsetAsync(e->d_ts.p, 0, sizeof(int), s));
    CK(cudaMemsetAsync(e->d_eacc.p, 0, 2 * sizeof(double), s));
    CK(cudaMemsetAsync(e->d_nsamp.p, 0, sizeof(int), s));
    CK(cudaMemsetAsync(e->d_err.p, 0, sizeof(int), s));
    e->ts = 0;
    e->need_initial_sample = true;
    return FDTD_OK;
}

// Operator::CreateEngine + Engine::Init for the CUDA engine: allocate the
// device arrays (fields start at zero) and copy the compressed operator.
int upload_engine(const fdtd_cop_s* c, const fdtd_engine_opts* opts, fdtd_engine_s* e) {
    for (int a = 0; a < 3; ++a) e->N[a] = c->N[a];
    e->dT = c->dT;
    e->device = opts ? opts->device : 0;
    CK(cudaSetDevice(e->device));
    CK(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking));
    CK(cudaEventCreate(&e->ev0));
    CK(cudaEventCreate(&e->ev1));
    e->TY = (opts && opts->tile_y > 0) ? opts->tile_y : 8;
    if (e->TY > 8 || e->TY < 1) {
        set_error("tile_y must be 1..8");
        return FDTD_ERR_ARG;
    }
    e->XC = (opts && opts->x_chunk > 0) ? opts->x_chunk : 16;
    e->interval = opts ? opts->probe_interval : 0;
    e->energy_on_probe = opts ? opts->energy_on_probe != 0 : true;
    e->use_graphs = opts ? opts->use_graphs != 0 : true;
    uint32_t maxts = (opts && opts->max_timesteps) ? opts->max_timesteps : 100000;
    e->cap = (e->interval ? maxts / e->interval : 0) + 2;
    e->num_tuples = c->num_tuples;
    e->upml_nodes = c->upml_nodes;
    e->ade_nodes = c->ade_nodes;
    e->idx16 = c->idx16;
    e->feat = c->feat;
    e->Nzp = c->Nzp;
    e->comp = c->comp;
    const uint32_t Nx = e->N[0], Ny = e->N[1], Nz = e->N[2];

    int rc;
    uint64_t& tot = e->device_bytes;
    const size_t F = 3 * (size_t)e->comp;
    if ((rc = e->V.alloc(F, tot)) || (rc = e->I.alloc(F, tot))) return rc;
    if (c->any_upml && ((rc = e->FV.alloc(F, tot)) || (rc = e->FI.alloc(F, tot)))) return rc;
    if (c->any_ade_e && (rc = e->AV.alloc(F, tot))) return rc;
    if (c->any_lor_e && (rc = e->LV.alloc(F, tot))) return rc;
    if (c->any_ade_h && (rc = e->AI.alloc(F, tot))) return rc;
    if (c->any_lor_h && (rc = e->LI.alloc(F, tot))) return rc;
    if ((rc = e->idx.alloc(c->idx_bytes, tot))) return rc;
    if ((rc = e->tabE.alloc(c->hE.size(), tot)) || (rc = e->tabH.alloc(c->hH.size(), tot)) ||
        (rc = e->tabEX.alloc(c->hEX.size(), tot)) || (rc = e->tabHX.alloc(c->hHX.size(), tot)))
        return rc;
    if (c->any_upml && ((rc = e->tabEU.alloc(c->hEU.size(), tot)) || (rc = e->tabHU.alloc(c->hHU.size(), tot))))
        return rc;
    if ((c->feat & FEAT_ADE) && ((rc = e->tabEA.alloc(c->hEA.size(), tot)) || (rc = e->tabHA.alloc(c->hHA.size(), tot))))
        return rc;
    uint32_t sl = std::max<uint32_t>(1, c->sig_len);
    if ((rc = e->sigV.alloc(sl, tot)) || (rc = e->sigC.alloc(sl, tot))) return rc;
    if ((rc = e->d_ts.alloc(1, tot)) || (rc = e->d_eacc.alloc(2, tot)) || (rc = e->d_energy_tmp.alloc(2, tot)) ||
        (rc = e->d_nsamp.alloc(1, tot)) || (rc = e->d_err.alloc(1, tot)))
        return rc;

    cudaStream_t s = e->stream;
    auto h2d = [&](void* dst, const void* src, size_t bytes) -> cudaError_t {
        return bytes ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s) : cudaSuccess;
    };
    CK(h2d(e->idx.p, c->idx, c->idx_bytes));
    CK(h2d(e->tabE.p, c->hE.data(), c->hE.size() * sizeof(float4)));
    CK(h2d(e->tabH.p, c->hH.data(), c->hH.size() * sizeof(float4)));
    CK(h2d(e->tabEX.p, c->hEX.data(), c->hEX.size() * sizeof(float4)));
    CK(h2d(e->tabHX.p, c->hHX.data(), c->hHX.size() * sizeof(float4)));
    if (c->any_upml) {
        CK(h2d(e->tabEU.p, c->hEU.data(), c->hEU.size() * sizeof(float4)));
        CK(h2d(e->tabHU.p, c->hHU.data(), c->hHU.size() * sizeof(float4)));
    }
    if (c->feat & FEAT_ADE) {
        CK(h2d(e->tabEA.p, c->hEA.data(), c->hEA.size() * sizeof(float4)));
        CK(h2d(e->tabHA.p, c->hHA.data(), c->hHA.size() * sizeof(float4)));
    }
    if (c->sig_len) {
        CK(h2d(e->sigV.p, c->sigV.data(), c->sig_len * sizeof(float)));
        CK(h2d(e->sigC.p, c->sigC.data(), c->sig_len * sizeof(float)));
    } else {
        CK(cudaMemsetAsync(e->sigV.p, 0, sizeof(float), s));
        CK(cudaMemsetAsync(e->sigC.p, 0, sizeof(float), s));
    }

    DevGrid& g = e->g;
    g.Nx = (int)Nx;
    g.Ny = (int)Ny;
    g.Nz = (int)Nz;
    g.Nzp = e->Nzp;
    g.sx = (long long)Ny * e->Nzp;
    g.comp = e->comp;
    g.V = e->V.p;
    g.I = e->I.p;
    g.FV = e->FV.p;
    g.FI = e->FI.p;
    g.AV = e->AV.p;
    g.LV = e->LV.p;
    g.AI = e->AI.p;
    g.LI = e->LI.p;
    g.idx = e->idx.p;
    g.tabE = e->tabE.p;
    g.tabH = e->tabH.p;
    g.tabEU = e->tabEU.p;
    g.tabHU = e->tabHU.p;
    g.tabEA = e->tabEA.p;
    g.tabHA = e->tabHA.p;
    g.tabEX = e->tabEX.p;
    g.tabHX = e->tabHX.p;
    g.sigV = e->sigV.p;
    g.sigC = e->sigC.p;
    g.sig_len = (int)c->sig_len;
    g.sig_period = (int)c->sig_period;
    g.d_ts = e->d_ts.p;
    g.d_eacc = e->d_eacc.p;
    e->smem_bytes = 2 * 3 * (size_t)(e->TY + 1) * 33 * sizeof(float);
    e->use_tma = !(opts && opts->kernel == 1);
    e->stages = (opts && opts->stages > 0) ? opts->stages : 3;
    e->zw = (opts && opts->z_per_thread > 0) ? opts->z_per_thread : 2;
    if (e->zw != 1 && e->zw != 2) {
        set_error("z_per_thread must be 1 or 2");
        return FDTD_ERR_ARG;
    }
    if (e->stages < 3 || e->stages > TMA_MAX_STAGES) {
        set_error("stages must be 3..8");
        return FDTD_ERR_ARG;
    }
    if (e->use_tma) {
        // opt in to more than 48 KB of dynamic shared memory where needed
        const size_t need = (e->feat & FEAT_UPML) ? StageLayout<uint32_t, true, 2>::smem(e->stages)
                                                  : StageLayout<uint32_t, false, 2>::smem(e->stages);
        if (need > 48 * 1024) {
            if ((rc = set_smem_attrs((int)need))) return rc;
        }
    }
    for (int a = 0; a < 3; ++a) {
        e->ti.lo[a] = c->inner_lo[a];
        e->ti.hi[a] = c->inner_hi[a];
        e->ti.ne[a] = (int)e->N[a] - (c->trim_e[a] ? 1 : 0);
    }
    e->ti.d_err = e->d_err.p;
    if (e->use_tma && (rc = make_maps(e))) return rc;
    return reset_state(e);
}

// Probe entries for ProcessVoltage (Engine_Interface_FDTD::CalcVoltageIntegral,
// engine_interface_fdtd.cpp:200-226) and ProcessCurrent::CalcIntegral
// (processcurrent.cpp:93-168), as (component, node, sign) lists.
int probe_entries(const fdtd_engine_s* e, const fdtd_probe_desc* p, std::vector<ProbeEntry>& out) {
    auto add = [&](int field, int comp, uint32_t x, uint32_t y, uint32_t z, int sign) -> int {
        if (x >= e->N[0] || y >= e->N[1] || z >= e->N[2]) {
            set_error("probe position outside the grid");
            return FDTD_ERR_ARG;
        }
        ProbeEntry pe;
        pe.off = (uint32_t)((long long)x * e->g.sx + (long long)y * e->Nzp + z);
        pe.comp = (int8_t)comp;
        pe.sign = (int8_t)sign;
        pe.field = (int8_t)field;
        pe.pad = 0;
        out.push_back(pe);
        return FDTD_OK;
    };
    if (!p->enabled) return FDTD_OK;
    const uint32_t* start = p->start;
    const uint32_t* stop = p->stop;
    if (p->type == 0) {
        int dims = (start[0] != stop[0]) + (start[1] != stop[1]) + (start[2] != stop[2]);
        if (dims != 1) return FDTD_OK;  // the reference prints an error and returns 0
        for (int n = 0; n < 3; ++n) {
            if (start[n] < stop[n]) {
                uint32_t pos[3] = {start[0], start[1], start[2]};
                for (; pos[n] < stop[n]; ++pos[n])
                    if (int rc = add(0, n, pos[0], pos[1], pos[2], +1)) return rc;
            } else {
                uint32_t pos[3] = {stop[0], stop[1], stop[2]};
                for (; pos[n] < start[n]; ++pos[n])
                    if (int rc = add(0, n, pos[0], pos[1], pos[2], -1)) return rc;
            }
        }
        return FDTD_OK;
    }
    const int* si = p->start_inside;
    const int* so = p->stop_inside;
    int rc = FDTD_OK;
    switch (p->norm_dir) {
        case 0:
            if (so[0] && si[2])
                for (uint32_t i = start[1] + 1; i <= stop[1] && !rc; ++i) rc = add(1, 1, stop[0], i, start[2], +1);
            if (so[0] && so[1])
                for (uint32_t i = start[2] + 1; i <= stop[2] && !rc; ++i) rc = add(1, 2, stop[0], stop[1], i, +1);
            if (si[0] && so[2])
                for (uint32_t i = start[1] + 1; i <= stop[1] && !rc; ++i) rc = add(1, 1, start[0], i, stop[2], -1);
            if (si[0] && si[1])
                for (uint32_t i = start[2] + 1; i <= stop[2] && !rc; ++i) rc = add(1, 2, start[0], start[1], i, -1);
            break;
        case 1:
            if (si[0] && si[1])
                for (uint32_t i = start[2] + 1; i <= stop[2] && !rc; ++i) rc = add(1, 2, start[0], start[1], i, +1);
            if (so[1] && so[2])
                for (uint32_t i = start[0] + 1; i <= stop[0] && !rc; ++i) rc = add(1, 0, i, stop[1], stop[2], +1);
            if (so[0] && so[1])
                for (uint32_t i = start[2] + 1; i <= stop[2] && !rc; ++i) rc = add(1, 2, stop[0], stop[1], i, -1);
            if (si[1] && si[2])
                for (uint32_t i = start[0] + 1; i <= stop[0] && !rc; ++i) rc = add(1, 0, i, start[1], start[2], -1);
            break;
        case 2:
            if (si[1] && si[2])
                for (uint32_t i = start[0] + 1; i <= stop[0] && !rc; ++i) rc = add(1, 0, i, start[1], start[2], +1);
            if (so[0] && si[2])
                for (uint32_t i = start[1] + 1; i <= stop[1] && !rc; ++i) rc = add(1, 1, stop[0], i, start[2], +1);
            if (so[1] && so[2])
                for (uint32_t i = start[0] + 1; i <= stop[0] && !rc; ++i) rc = add(1, 0, i, stop[1], stop[2], -1);
            if (si[0] && so[2])
                for (uint32_t i = start[1] + 1; i <= stop[1] && !rc; ++i) rc = add(1, 1, start[0], i, stop[2], -1);
            break;
        default:
            break;
    }
    return rc;
}

}  // namespace
}  // namespace wipems

// ===================================================================== C ABI
extern "C" {

int fdtd_compress(const fdtd_op_desc* desc, fdtd_cop_t* out) {
    if (!desc || !out) {
        set_error("fdtd_compress: null argument");
        return FDTD_ERR_ARG;
    }
    fdtd_cop_s* c = new (std::nothrow) fdtd_cop_s();
    if (!c) return FDTD_ERR_NOMEM;
    int rc;
    try {
        rc = compress_op(desc, c);
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

int fdtd_cop_destroy(fdtd_cop_t c) {
    delete c;
    return FDTD_OK;
}

int fdtd_cop_get_info(fdtd_cop_t c, fdtd_cop_info* info) {
    if (!c || !info) return FDTD_ERR_ARG;
    std::memset(info, 0, sizeof(*info));
    for (int a = 0; a < 3; ++a) info->num_lines[a] = c->N[a];
    info->num_tuples = c->num_tuples;
    info->index_bytes = c->idx16 ? 2 : 4;
    info->padded_nz = (uint32_t)c->Nzp;
    info->num_upml_nodes = c->upml_nodes;
    info->num_ade_nodes = c->ade_nodes;
    info->host_bytes = c->idx_bytes + (c->hE.size() + c->hH.size() + c->hEU.size() + c->hHU.size() + c->hEA.size() +
                                       c->hHA.size() + c->hEX.size() + c->hHX.size()) * sizeof(float4);
    info->pinned = c->idx_pinned ? 1 : 0;
    return FDTD_OK;
}

int fdtd_cop_expand(fdtd_cop_t c, float* vv, float* vi, float* ii, float* iv, uint32_t* flags_e, uint32_t* flags_h) {
    if (!c) return FDTD_ERR_ARG;
    const uint32_t Nx = c->N[0], Ny = c->N[1], Nz = c->N[2];
    const size_t NN = (size_t)Nx * Ny * Nz;
    for (uint32_t x = 0; x < Nx; ++x)
        for (uint32_t y = 0; y < Ny; ++y)
            for (uint32_t z = 0; z < Nz; ++z) {
                const size_t pi = ((size_t)x * Ny + y) * c->Nzp + z;
                const uint32_t t = c->idx16 ? reinterpret_cast<const uint16_t*>(c->idx)[pi]
                                            : reinterpret_cast<const uint32_t*>(c->idx)[pi];
                const float* e = reinterpret_cast<const float*>(&c->hE[2 * (size_t)t]);
                const float* h = reinterpret_cast<const float*>(&c->hH[2 * (size_t)t]);
                const size_t gi = ((size_t)x * Ny + y) * Nz + z;
                for (int n = 0; n < 3; ++n) {
                    if (vv) vv[n * NN + gi] = e[n];
                    if (vi) vi[n * NN + gi] = e[3 + n];
                    if (ii) ii[n * NN + gi] = h[n];
                    if (iv) iv[n * NN + gi] = h[3 + n];
                }
                if (flags_e) std::memcpy(&flags_e[gi], &e[6], 4);
                if (flags_h) std::memcpy(&flags_h[gi], &h[6], 4);
            }
    return FDTD_OK;
}

int fdtd_engine_create_compressed(fdtd_cop_t cop, const fdtd_engine_opts* opts, fdtd_engine_t* out) {
    if (!cop || !out) {
        set_error("fdtd_engine_create_compressed: null argument");
        return FDTD_ERR_ARG;
    }
    fdtd_engine_s* e = new (std::nothrow) fdtd_engine_s();
    if (!e) return FDTD_ERR_NOMEM;
    int rc = upload_engine(cop, opts, e);
    if (rc == FDTD_OK) {
        cudaError_t ce = cudaStreamSynchronize(e->stream);
        if (ce != cudaSuccess) {
            set_error(std::string("engine upload: ") + cudaGetErrorString(ce));
            rc = FDTD_ERR_CUDA;
        }
    }
    if (rc != FDTD_OK) {
        delete e;
        return rc;
    }
    *out = e;
    return FDTD_OK;
}

int fdtd_engine_create(const fdtd_op_desc* desc, const fdtd_engine_opts* opts, fdtd_engine_t* out) {
    fdtd_cop_t c = nullptr;
    int rc = fdtd_compress(desc, &c);
    if (rc) return rc;
    rc = fdtd_engine_create_compressed(c, opts, out);
    fdtd_cop_destroy(c);
    return rc;
}

int fdtd_engine_reset(fdtd_engine_t e) {
    if (!e) return FDTD_ERR_ARG;
    CK(cudaSetDevice(e->device));
    return reset_state(e);
}

int fdtd_engine_destroy(fdtd_engine_t e) {
    if (!e) return FDTD_OK;
    cudaSetDevice(e->device);
    if (e->stream) cudaStreamSynchronize(e->stream);
    delete e;
    return FDTD_OK;
}

int fdtd_engine_add_probe(fdtd_engine_t e, const fdtd_probe_desc* p, uint32_t* slot) {
    if (!e || !p) return FDTD_ERR_ARG;
    if (e->started) {
        set_error("fdtd_engine_add_probe: probes must be added before the first iterate");
        return FDTD_ERR_STATE;
    }
    std::vector<ProbeEntry> ent;
    int rc = probe_entries(e, p, ent);
    if (rc) return rc;
    e->h_entries.insert(e->h_entries.end(), ent.begin(), ent.end());
    e->h_first.push_back((int)e->h_entries.size());
    e->h_weight.push_back(p->weight);
    if (slot) *slot = (uint32_t)(e->h_weight.size() - 1);
    return FDTD_OK;
}

int fdtd_engine_iterate(fdtd_engine_t e, uint32_t n) {
    if (!e) return FDTD_ERR_ARG;
    CK(cudaSetDevice(e->device));
    e->last_launches = 0;
    int rc;
    if (!e->started) {
        if ((rc = upload_probes(e))) return rc;
        e->started = true;
        if (e->interval && e->use_graphs && (rc = build_chunk_graph(e))) return rc;
    }
    CK(cudaEventRecord(e->ev0, e->stream));
    if (e->need_initial_sample) {
        e->need_initial_sample = false;
        if (e->interval) {  // sample at ts = 0 (RunFDTD's PA->Process() before the loop)
            if ((rc = launch_advance(e, 0, true, e->energy_on_probe))) return rc;
        }
    }
    uint32_t left = n;
    while (left > 0) {
        if (e->interval && e->use_graphs && e->chunk && (e->ts % e->interval) == 0 && left >= e->interval) {
            CK(cudaGraphLaunch(e->chunk, e->stream));
            e->last_launches += 2 * (uint64_t)e->interval + 1;
            e->ts += e->interval;
            left -= e->interval;
            continue;
        }
        bool sample = e->interval && ((e->ts + 1) % e->interval) == 0;
        if ((rc = launch_step(e, 0, sample && e->energy_on_probe))) return rc;
        if ((rc = launch_advance(e, 1, sample, e->energy_on_probe))) return rc;
        e->ts += 1;
        left -= 1;
    }
    CK(cudaEventRecord(e->ev1, e->stream));
    CK(cudaEventSynchronize(e->ev1));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, e->ev0, e->ev1));
    e->last_ms = ms;
    int err = 0;
    CK(cudaMemcpy(&err, e->d_err.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (err & 1) {
        set_error("probe sample ring overflow: raise max_timesteps");
        return FDTD_ERR_STATE;
    }
    if (err & 4) {
        set_error("a bounded device wait gave up: a TMA copy did not complete in time");
        return FDTD_ERR_TIMEOUT;
    }
    if (err & 2) {
        set_error("energy reduction is not finite (NaN/Inf in the fields)");
        return FDTD_ERR_NONFINITE;
    }
    return FDTD_OK;
}

int fdtd_engine_num_timesteps(fdtd_engine_t e, uint32_t* ts) {
    if (!e || !ts) return FDTD_ERR_ARG;
    *ts = e->ts;
    return FDTD_OK;
}

int fdtd_engine_num_samples(fdtd_engine_t e, uint32_t* n) {
    if (!e || !n) return FDTD_ERR_ARG;
    if (!e->started) {
        *n = 0;
        return FDTD_OK;
    }
    CK(cudaSetDevice(e->device));
    int v = 0;
    CK(cudaMemcpyAsync(&v, e->d_nsamp.p, sizeof(int), cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    *n = (uint32_t)v;
    return FDTD_OK;
}

int fdtd_engine_read_samples(fdtd_engine_t e, uint32_t first, uint32_t count, uint32_t* ts, double* vals,
                             double* energy) {
    if (!e) return FDTD_ERR_ARG;
    uint32_t n = 0;
    int rc = fdtd_engine_num_samples(e, &n);
    if (rc) return rc;
    if (first + count > n) {
        set_error("fdtd_engine_read_samples: range beyond recorded samples");
        return FDTD_ERR_ARG;
    }
    if (count == 0) return FDTD_OK;
    const int row = e->ps.row_doubles;
    std::vector<double> buf((size_t)count * row);
    CK(cudaMemcpyAsync(buf.data(), e->ring.p + (size_t)first * row, buf.size() * sizeof(double),
                       cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    const int np = e->ps.nprobe;
    for (uint32_t k = 0; k < count; ++k) {
        const double* r = &buf[(size_t)k * row];
        if (ts) ts[k] = (uint32_t)r[0];
        if (energy) energy[k] = r[1];
        if (vals)
            for (int p = 0; p < np; ++p) vals[(size_t)k * np + p] = r[2 + p];
    }
    return FDTD_OK;
}

int fdtd_engine_energy(fdtd_engine_t e, double* energy) {
    if (!e || !energy) return FDTD_ERR_ARG;
    CK(cudaSetDevice(e->device));
    CK(cudaMemsetAsync(e->d_energy_tmp.p, 0, 2 * sizeof(double), e->stream));
    k_energy<<<4 * 152, 256, 0, e->stream>>>(e->g, e->d_energy_tmp.p);
    CK(cudaGetLastError());
    double h[2];
    CK(cudaMemcpyAsync(h, e->d_energy_tmp.p, sizeof(h), cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    *energy = kEps0 * h[0] + kMue0 * h[1];
    return FDTD_OK;
}

int fdtd_engine_get_fields(fdtd_engine_t e, float* volt, float* curr) {
    if (!e) return FDTD_ERR_ARG;
    CK(cudaSetDevice(e->device));
    const uint32_t Nx = e->N[0], Ny = e->N[1], Nz = e->N[2];
    for (int which = 0; which < 2; ++which) {
        float* dst = which ? curr : volt;
        if (!dst) continue;
        const float* src = which ? e->I.p : e->V.p;
        // strided 3-D copy: rows of Nz floats out of rows of Nzp floats
        CK(cudaMemcpy2DAsync(dst, Nz * sizeof(float), src, e->Nzp * sizeof(float), Nz * sizeof(float),
                             (size_t)3 * Nx * Ny, cudaMemcpyDeviceToHost, e->stream));
    }
    CK(cudaStreamSynchronize(e->stream));
    return FDTD_OK;
}

static int get_one(fdtd_engine_t e, const float* base, uint32_t n, uint32_t x, uint32_t y, uint32_t z, float* v) {
    if (!e || !v || n > 2 || x >= e->N[0] || y >= e->N[1] || z >= e->N[2]) {
        set_error("field access out of range");
        return FDTD_ERR_ARG;
    }
    CK(cudaSetDevice(e->device));
    long long off = n * e->comp + (long long)x * e->g.sx + (long long)y * e->Nzp + z;
    CK(cudaMemcpyAsync(v, base + off, sizeof(float), cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    return FDTD_OK;
}

int fdtd_engine_get_volt(fdtd_engine_t e, uint32_t n, uint32_t x, uint32_t y, uint32_t z, float* v) {
    return get_one(e, e ? e->V.p : nullptr, n, x, y, z, v);
}
int fdtd_engine_get_curr(fdtd_engine_t e, uint32_t n, uint32_t x, uint32_t y, uint32_t z, float* v) {
    return get_one(e, e ? e->I.p : nullptr, n, x, y, z, v);
}

int fdtd_engine_profile_kernels(fdtd_engine_t e, uint32_t n_steps, double* ms_volt, double* ms_curr) {
    if (!e || n_steps == 0) return FDTD_ERR_ARG;
    CK(cudaSetDevice(e->device));
    int rc;
    if (!e->started) {
        if ((rc = upload_probes(e))) return rc;
        e->started = true;
        if (e->interval && e->use_graphs && (rc = build_chunk_graph(e))) return rc;
    }
    if (e->need_initial_sample) {
        e->need_initial_sample = false;
        if (e->interval && (rc = launch_advance(e, 0, true, e->energy_on_probe))) return rc;
    }
    std::vector<cudaEvent_t> ev(3 * (size_t)n_steps);
    for (auto& x : ev) CK(cudaEventCreate(&x));
    dim3 block(32, e->TY);
    dim3 gv((e->N[2] + 31) / 32, (e->N[1] + e->TY - 1) / e->TY, (e->N[0] + e->XC - 1) / e->XC);
    dim3 gc((e->N[2] + 31) / 32, (e->N[1] + e->TY - 1) / e->TY, (e->N[0] - 1 + e->XC - 1) / e->XC);
    for (uint32_t k = 0; k < n_steps; ++k) {
        bool sample = e->interval && ((e->ts + 1) % e->interval) == 0;
        bool energy = sample && e->energy_on_probe;
        VoltFn fv = e->idx16 ? pick_volt<uint16_t>(e->feat) : pick_volt<uint32_t>(e->feat);
        CurrFn fc = e->idx16 ? pick_curr<uint16_t>(e->feat, energy) : pick_curr<uint32_t>(e->feat, energy);
        CK(cudaEventRecord(ev[3 * k], e->stream));
        if (e->use_tma) {
            // volt then curr with an event in between
            if (e->idx16)
                launch_tma_half<uint16_t>(e, 0, energy, true);
            else
                launch_tma_half<uint32_t>(e, 0, energy, true);
        } else {
            fv<<<gv, block, e->smem_bytes, e->stream>>>(e->g, 0, e->XC);
        }
        CK(cudaEventRecord(ev[3 * k + 1], e->stream));
        if (e->use_tma) {
            if (e->idx16)
                launch_tma_half<uint16_t>(e, 0, energy, false);
            else
                launch_tma_half<uint32_t>(e, 0, energy, false);
        } else {
            fc<<<gc, block, e->smem_bytes, e->stream>>>(e->g, 0, e->XC);
        }
        CK(cudaEventRecord(ev[3 * k + 2], e->stream));
        CK(cudaGetLastError());
        if ((rc = launch_advance(e, 1, sample, e->energy_on_probe))) return rc;
        e->ts += 1;
    }
    CK(cudaStreamSynchronize(e->stream));
    double sv = 0, sc = 0;
    for (uint32_t k = 0; k < n_steps; ++k) {
        float a = 0, b = 0;
        CK(cudaEventElapsedTime(&a, ev[3 * k], ev[3 * k + 1]));
        CK(cudaEventElapsedTime(&b, ev[3 * k + 1], ev[3 * k + 2]));
        sv += a;
        sc += b;
    }
    for (auto& x : ev) cudaEventDestroy(x);
    if (ms_volt) *ms_volt = sv / n_steps;
    if (ms_curr) *ms_curr = sc / n_steps;
    return FDTD_OK;
}

int fdtd_engine_get_stats(fdtd_engine_t e, fdtd_engine_stats* st) {
    if (!e || !st) return FDTD_ERR_ARG;
    std::memset(st, 0, sizeof(*st));
    st->num_tuples = e->num_tuples;
    st->index_bytes = e->idx16 ? 2 : 4;
    st->num_upml_nodes = e->upml_nodes;
    st->num_ade_nodes = e->ade_nodes;
    st->padded_nz = (uint32_t)e->Nzp;
    st->device_bytes = e->device_bytes;
    st->tile_y = (uint32_t)e->TY;
    st->x_chunk = (uint32_t)e->XC;
    return FDTD_OK;
}

int fdtd_engine_last_timing(fdtd_engine_t e, double* ms, uint64_t* launches) {
    if (!e) return FDTD_ERR_ARG;
    if (ms) *ms = e->last_ms;
    if (launches) *launches = e->last_launches;
    return FDTD_OK;
}

}  // extern "C"
