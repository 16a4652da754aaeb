// Internal state of Engine_CUDA shared by engine.cu and batch.cu (not part
// of the C ABI).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "cop.h"
#include "fdtd_host.h"
#include "kernels.cuh"
#include "kernels_fused.cuh"
#include "kernels_tma.cuh"

namespace wipems {

#define CK(call)                                                           \
    do {                                                                   \
        cudaError_t e_ = (call);                                           \
        if (e_ != cudaSuccess) {                                           \
            set_error(std::string(#call) + ": " + cudaGetErrorString(e_)); \
            return FDTD_ERR_CUDA;                                          \
        }                                                                  \
    } while (0)

// Device buffer.  With a stream the memory comes from the device's
// stream-ordered pool (cudaMallocAsync / cudaFreeAsync on that stream):
// unlike cudaMalloc / cudaFree, neither synchronises the device, so a
// server can create and destroy engines while other engines' work is in
// flight.  The stream must outlive the buffer.
template <class T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    cudaStream_t s = nullptr;
    ~DevBuf() { release(); }
    void release() {
        if (p) {
            if (s) cudaFreeAsync(p, s);
            else cudaFree(p);
        }
        p = nullptr;
    }
    int alloc(size_t count, uint64_t& total, cudaStream_t stream = nullptr) {
        n = count;
        s = stream;
        if (count == 0) return FDTD_OK;
        cudaError_t e = stream ? cudaMallocAsync(&p, count * sizeof(T), stream) : cudaMalloc(&p, count * sizeof(T));
        if (e == cudaSuccess && stream) e = cudaStreamSynchronize(stream);  // usable from any stream from here on
        if (e != cudaSuccess) {
            p = nullptr;
            set_error(std::string(stream ? "cudaMallocAsync: " : "cudaMalloc: ") + cudaGetErrorString(e));
            return FDTD_ERR_NOMEM;
        }
        total += count * sizeof(T);
        return FDTD_OK;
    }
};

struct DevHalfBufs {
    DevBuf<uint8_t> idx;
    DevBuf<float> main, upml, ade, exc, adex;
    bool idx16 = true;
};

}  // namespace wipems

using namespace wipems;

struct fdtd_engine_s {
    int device = 0;
    cudaStream_t stream = nullptr;
    // destroys the stream after every member declared below (the device
    // buffers free themselves on it first)
    struct StreamGuard {
        cudaStream_t* s;
        ~StreamGuard() {
            if (*s) cudaStreamDestroy(*s);
        }
    } stream_guard{&stream};
    uint32_t N[3];             // device axes (see fdtd_cop_s)
    uint32_t N0[3] = {0, 0, 0};  // the operator's axes, in which the API speaks
    int rot = 0;               // device axis a = operator axis (a + rot) % 3
    int Nzp = 0;
    // device node / component of a node / component in the operator's axes
    void dev_node(const uint32_t o[3], uint32_t d[3]) const {
        for (int a = 0; a < 3; ++a) d[a] = o[(a + rot) % 3];
    }
    int dev_comp(int n) const { return (n - rot + 3) % 3; }
    long long dev_offset(const uint32_t o[3]) const {
        uint32_t d[3];
        dev_node(o, d);
        return (long long)d[0] * g.sx + (long long)d[1] * Nzp + d[2];
    }
    long long comp = 0;
    double dT = 0;
    DevGrid g{};
    DevBuf<float> V, I, FV, FI, AV, LV, AI, LI;
    DevBuf<float> AVx, LVx, AIx, LIx;  // states of dispersion orders 1..3: [order-1][3][comp]
    DevBuf<uint8_t> ade_tile;  // per voltage-kernel tile plane: Lorentz/Drude flags (DevGrid::ade_tile)
    DevBuf<double> edges;      // [2][Nx+Ny+Nz] main / dual edge lengths (field dumps; empty = no mesh lines)
    DevBuf<float> dump;        // field-dump scratch, grown on demand
    DevBuf<float> V2, I2, FV2;  // second field / voltage-flux buffers (fused kernel)
    DevHalfBufs E, H;
    DevBuf<float> geo;
    DevBuf<float> sigV, sigC;
    // control words, one allocation so a single copy reads them all:
    // [0] numTS, [1] samples recorded, [2] error word, [3] done flag
    DevBuf<int> ctl;
    int* p_ts() const { return ctl.p; }
    int* p_nsamp() const { return ctl.p + 1; }
    int* p_err() const { return ctl.p + 2; }
    int* p_done() const { return ctl.p + 3; }
    DevBuf<double> d_eacc;  // [2]: running energy maximum (end criterion)
    DevBuf<double> d_energy_tmp;
    DevBuf<ProbeEntry> now_entries;  // fdtd_engine_probe_now scratch, grown on demand
    DevBuf<double> now_misc;
    DevBuf<float2> eseg;    // energy segments (DevGrid::eseg)
    DevBuf<double2> eplane; // energy plane sums (DevGrid::eplane)
    // probes
    std::vector<ProbeEntry> h_entries;
    std::vector<int> h_first{0};
    std::vector<double> h_weight;
    std::vector<double> h_div;         // per column: 0 integral, else field-probe edge length (see ProbeSet::div)
    std::vector<double> h_edges;       // host copy of the edge lengths (field probes)
    std::vector<int> h_dual;           // per probe: 1 = current probe (dual time)
    // frequency-domain accumulation (0 frequencies = off)
    std::vector<double> h_freq;
    uint32_t fd_interval = 0;
    DevBuf<double> d_freq, d_fd;
    DevBuf<int> d_fd_dual, d_fd_count;
    FdSet fd{};
    // Mur ABC faces
    DevBuf<float> mur_coef, mur_buf;
    MurSet mur{};
    // lumped RLC edges
    DevBuf<float> rlc_coef, rlc_state;
    DevBuf<long long> rlc_off;
    RlcSet rlc{};
    DevBuf<ProbeEntry> d_entries;
    DevBuf<int> d_first;
    DevBuf<double> d_weight, d_div;
    DevBuf<double> ring;
    ProbeSet ps{};
    bool probes_uploaded = false;
    uint32_t interval = 0;
    bool energy_on_probe = true;
    bool use_graphs = true;
    bool pending = false;    // an asynchronous iterate was launched, not yet waited for
    double end_crit = 0;     // > 0: stop on the device (energy decay or stop_ts)
    uint32_t stop_ts = 0;
    bool done = false;       // as of the last control-word read
    uint32_t cap = 0;
    // state
    uint32_t ts = 0;
    bool started = false;
    bool need_initial_sample = true;
    int feat = 0;                // union of the two halves' feature sets
    int feat_e = 0, feat_h = 0;  // the voltage / current kernels' feature sets (FEAT_*)
    bool geo_on = false;
    int TY = 8;       // direct kernels: tile rows
    int tma_ty = 4;   // two-pass TMA kernels: tile rows (4 or 8)
    int XC = 8;
    bool use_tma = true;
    bool fused = false;      // single-pass kernel, double-buffered fields
    FusedMaps fmaps{};
    // field buffers holding the fields at the current numTS
    float* cur_V() const { return (fused && (ts & 1)) ? V2.p : V.p; }
    float* cur_I() const { return (fused && (ts & 1)) ? I2.p : I.p; }
    int stages = 3;
    TmaMaps maps{};
    TileInfo ti{};
    size_t smem_direct = 0;
    uint32_t num_tuples_e = 0, num_tuples_h = 0, upml_nodes = 0, ade_nodes = 0;
    uint64_t device_bytes = 0;
    cudaGraphExec_t chunk = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    double last_ms = 0;
    uint64_t last_launches = 0;

    ~fdtd_engine_s() {
        if (chunk) cudaGraphExecDestroy(chunk);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
    }
};


namespace wipems {
// x-chunk (planes per block: 1, 2, 4, 8 or 16) from a wave model of the
// current-kernel grid: a block costs about (2 + x_chunk) plane times (the
// ring prologue, then one plane each), blocks run in waves of `resident`,
// so the step costs ceil(blocks / resident) * (2 + x_chunk); a chunk that
// leaves SMs idle in the only wave is skipped, ties go to the longer chunk
// (fewer halo-plane re-reads).  lines: the jobs' (Nx, Ny, Nz) triples.
inline int auto_x_chunk(const std::vector<const uint32_t*>& lines, uint64_t resident, int ty = TMA_TY) {
    int best = 1;
    uint64_t best_cost = ~0ull;
    for (int xc = 16; xc >= 1; xc /= 2) {
        uint64_t items = 0;
        for (const uint32_t* N : lines)
            items += (uint64_t)((N[2] - 1 + 31) / 32) * ((N[1] - 1 + ty - 1) / ty) * ((N[0] - 1 + xc - 1) / xc);
        if (items < resident && xc > 1) continue;
        const uint64_t cost = (items + resident - 1) / resident * (uint64_t)(2 + xc);
        if (cost < best_cost) {
            best_cost = cost;
            best = xc;
        }
    }
    return best;
}

// engine.cu helpers used by the batched path
int engine_start(fdtd_engine_s* e);        // upload probes, graph, ts = 0 sample
int engine_tma_maps(const fdtd_engine_s* e, TmaMaps* out, uint32_t rows);  // tensor maps for rows-high tiles
int engine_check_errors(fdtd_engine_s* e); // read the control words, decode errors
int engine_decode_error(int err);          // error word -> status code + message
}  // namespace wipems
