// Engine_CUDA: the device-resident FDTD time stepper behind the C ABI.
//
// fdtd_engine_create_compressed plays the part of Operator::CreateEngine +
// Engine::Init (FDTD/operator.cpp:63-67, FDTD/engine.cpp:49-57) for the CUDA
// engine: it allocates the zeroed field arrays and copies the compressed
// operator (compress.cpp) to the device.  fdtd_engine_iterate is
// Engine::IterateTS (engine.cpp:255-274): per timestep one voltage and one
// current kernel, with probe sampling and the energy reduction at the probe
// interval; chunks of one probe interval are captured once into a CUDA graph
// and replayed.
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>


#include "engine_state.h"
#include "launch.cuh"

namespace wipems {
namespace {

// ------------------------------------------------------------ kernel launch
// (the per-variant launch templates are in launch.cuh; the variants with
// dispersion orders 1..3 are instantiated in engine_adex.cu)
template <typename IdxT, bool GEO>
void launch_volt_f(fdtd_engine_s* e, int ts_off) {
    switch (e->feat_e) {
        case 0: launch_volt_t<IdxT, 0, GEO>(e, ts_off); break;
        case 1: launch_volt_t<IdxT, 1, GEO>(e, ts_off); break;
        case 2: launch_volt_t<IdxT, 2, GEO>(e, ts_off); break;
        case 3: launch_volt_t<IdxT, 3, GEO>(e, ts_off); break;
        default: launch_volt_adex<IdxT, GEO>(e, ts_off); break;
    }
}

template <typename IdxT, bool GEO, bool EN>
void launch_curr_f(fdtd_engine_s* e, int ts_off) {
    switch (e->feat_h) {
        case 0: launch_curr_t<IdxT, 0, GEO, EN>(e, ts_off); break;
        case 1: launch_curr_t<IdxT, 1, GEO, EN>(e, ts_off); break;
        case 2: launch_curr_t<IdxT, 2, GEO, EN>(e, ts_off); break;
        case 3: launch_curr_t<IdxT, 3, GEO, EN>(e, ts_off); break;
        default: launch_curr_adex<IdxT, GEO, EN>(e, ts_off); break;
    }
}

void launch_volt(fdtd_engine_s* e, int ts_off) {
    if (e->E.idx16) {
        if (e->geo_on) launch_volt_f<uint16_t, true>(e, ts_off);
        else launch_volt_f<uint16_t, false>(e, ts_off);
    } else {
        if (e->geo_on) launch_volt_f<uint32_t, true>(e, ts_off);
        else launch_volt_f<uint32_t, false>(e, ts_off);
    }
}

void launch_curr(fdtd_engine_s* e, int ts_off, bool energy) {
    if (e->H.idx16) {
        if (e->geo_on) {
            if (energy) launch_curr_f<uint16_t, true, true>(e, ts_off);
            else launch_curr_f<uint16_t, true, false>(e, ts_off);
        } else {
            if (energy) launch_curr_f<uint16_t, false, true>(e, ts_off);
            else launch_curr_f<uint16_t, false, false>(e, ts_off);
        }
    } else {
        if (e->geo_on) {
            if (energy) launch_curr_f<uint32_t, true, true>(e, ts_off);
            else launch_curr_f<uint32_t, true, false>(e, ts_off);
        } else {
            if (energy) launch_curr_f<uint32_t, false, true>(e, ts_off);
            else launch_curr_f<uint32_t, false, false>(e, ts_off);
        }
    }
}

template <typename IE, typename IH, int FEAT, bool EN>
void launch_fused_t(fdtd_engine_s* e, int ts_off) {
    const size_t sm = FusedLayout<IE, IH, (FEAT & FEAT_UPML) != 0>::smem(e->stages);
    dim3 grid((e->N[2] - 1 + 31) / 32, (e->N[1] - 1 + FU_TY - 1) / FU_TY, (e->N[0] - 1 + e->XC - 1) / e->XC);
    k_step_fused<IE, IH, FEAT, EN><<<grid, dim3(32, FU_WARPS), sm, e->stream>>>(e->g, e->fmaps, e->ti, ts_off, e->XC,
                                                                             e->stages);
}
template <typename IE, typename IH, bool EN>
void launch_fused_f(fdtd_engine_s* e, int ts_off) {
    if (e->feat & FEAT_UPML) launch_fused_t<IE, IH, FEAT_UPML, EN>(e, ts_off);
    else launch_fused_t<IE, IH, 0, EN>(e, ts_off);
}
template <bool EN>
void launch_fused_e(fdtd_engine_s* e, int ts_off) {
    if (e->E.idx16) {
        if (e->H.idx16) launch_fused_f<uint16_t, uint16_t, EN>(e, ts_off);
        else launch_fused_f<uint16_t, uint32_t, EN>(e, ts_off);
    } else {
        if (e->H.idx16) launch_fused_f<uint32_t, uint16_t, EN>(e, ts_off);
        else launch_fused_f<uint32_t, uint32_t, EN>(e, ts_off);
    }
}
void launch_fused(fdtd_engine_s* e, int ts_off, bool energy) {
    if (energy) launch_fused_e<true>(e, ts_off);
    else launch_fused_e<false>(e, ts_off);
}

int check_launch() {
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) {
        set_error(std::string("kernel launch: ") + cudaGetErrorString(err));
        return FDTD_ERR_CUDA;
    }
    return FDTD_OK;
}

void launch_mur(fdtd_engine_s* e, int ts_off, int stage) {
    const unsigned blocks = std::min<unsigned>((e->mur.total + 255) / 256, 1024u);
    k_mur<<<blocks, 256, 0, e->stream>>>(e->g, e->mur, ts_off, stage);
    e->last_launches += 1;
}

void launch_rlc(fdtd_engine_s* e, int ts_off) {
    const unsigned blocks = std::min<unsigned>((e->rlc.count + 127) / 128, 1024u);
    k_rlc<<<blocks, 128, 0, e->stream>>>(e->g, e->rlc, ts_off);
    e->last_launches += 1;
}

// The voltage half-step with the passes that surround it: Mur pre-update,
// the voltage kernel, Mur post-update, lumped RLC, Mur apply (the
// reference's hook order for these extensions).
void launch_volt_hooks(fdtd_engine_s* e, int ts_off) {
    if (e->mur.nface) launch_mur(e, ts_off, 0);
    launch_volt(e, ts_off);
    if (e->mur.nface) launch_mur(e, ts_off, 1);
    if (e->rlc.count) launch_rlc(e, ts_off);
    if (e->mur.nface) launch_mur(e, ts_off, 2);
}

int launch_step(fdtd_engine_s* e, int ts_off, bool energy) {
    if (e->mur.nface || e->rlc.count) {
        launch_volt_hooks(e, ts_off);
        launch_curr(e, ts_off, energy);
        e->last_launches += 2;
        return check_launch();
    }
    if (e->fused) {
        launch_fused(e, ts_off, energy);
        e->last_launches += 1;
        return check_launch();
    }
    launch_volt(e, ts_off);
    launch_curr(e, ts_off, energy);
    e->last_launches += 2;
    return check_launch();
}

int launch_advance(fdtd_engine_s* e, int adv, bool sample, bool energy_valid) {
    if (sample && energy_valid && adv > 0) {  // the last current kernel wrote the energy segments
        k_energy_planes<<<e->N[0] - 1, 256, 0, e->stream>>>(e->g);
        e->last_launches += 1;
    }
    k_advance_sample<<<1, 256, 0, e->stream>>>(e->p_ts(), adv, sample ? 1 : 0, e->ps, e->g, energy_valid ? 1 : 0,
                                                kEps0, kMue0);
    e->last_launches += 1;
    return check_launch();
}

// frequency-domain accumulation at numTS = ts (after the step that reached it)
int launch_fd(fdtd_engine_s* e, uint32_t ts) {
    if (!e->fd_interval || e->h_freq.empty() || e->ps.nprobe == 0) return FDTD_OK;
    const size_t sm = std::max<size_t>(8, (size_t)e->ps.nprobe * sizeof(double));
    k_fd_accumulate<<<1, 256, sm, e->stream>>>(e->p_ts(), (int)ts, e->ps, e->g, e->fd);
    e->last_launches += 1;
    return check_launch();
}

// ------------------------------------------------------------------ probes
int upload_probes(fdtd_engine_s* e) {
    if (e->probes_uploaded) return FDTD_OK;
    const uint32_t np = (uint32_t)e->h_weight.size();
    int rc;
    if ((rc = e->d_entries.alloc(std::max<size_t>(1, e->h_entries.size()), e->device_bytes, e->stream))) return rc;
    if ((rc = e->d_first.alloc(np + 1, e->device_bytes, e->stream))) return rc;
    if ((rc = e->d_weight.alloc(std::max<uint32_t>(1, np), e->device_bytes, e->stream))) return rc;
    if ((rc = e->d_div.alloc(std::max<uint32_t>(1, np), e->device_bytes, e->stream))) return rc;
    if (!e->h_entries.empty())
        CK(cudaMemcpyAsync(e->d_entries.p, e->h_entries.data(), e->h_entries.size() * sizeof(ProbeEntry),
                           cudaMemcpyHostToDevice, e->stream));
    CK(cudaMemcpyAsync(e->d_first.p, e->h_first.data(), (np + 1) * sizeof(int), cudaMemcpyHostToDevice, e->stream));
    if (np) {
        CK(cudaMemcpyAsync(e->d_weight.p, e->h_weight.data(), np * sizeof(double), cudaMemcpyHostToDevice,
                           e->stream));
        CK(cudaMemcpyAsync(e->d_div.p, e->h_div.data(), np * sizeof(double), cudaMemcpyHostToDevice, e->stream));
    }
    const int row = 2 + (int)np;
    if ((rc = e->ring.alloc((size_t)e->cap * row, e->device_bytes, e->stream))) return rc;
    e->ps.entries = e->d_entries.p;
    e->ps.first = e->d_first.p;
    e->ps.weight = e->d_weight.p;
    e->ps.div = e->d_div.p;
    e->ps.nprobe = (int)np;
    e->ps.row_doubles = row;
    e->ps.ring = e->ring.p;
    e->ps.cap = (int)e->cap;
    e->ps.d_nsamp = e->p_nsamp();
    e->ps.d_err = e->p_err();
    e->ps.d_done = e->p_done();
    e->ps.end_crit = e->end_crit;
    e->ps.stop_ts = e->end_crit > 0 ? (int)e->stop_ts : 0;
    if (e->fd_interval && !e->h_freq.empty() && np) {
        const size_t nf = e->h_freq.size();
        uint64_t& tb = e->device_bytes;
        if ((rc = e->d_freq.alloc(nf, tb, e->stream)) || (rc = e->d_fd.alloc(2 * np * nf, tb, e->stream)) ||
            (rc = e->d_fd_dual.alloc(np, tb, e->stream)) || (rc = e->d_fd_count.alloc(1, tb, e->stream)))
            return rc;
        CK(cudaMemcpyAsync(e->d_freq.p, e->h_freq.data(), nf * sizeof(double), cudaMemcpyHostToDevice, e->stream));
        CK(cudaMemcpyAsync(e->d_fd_dual.p, e->h_dual.data(), np * sizeof(int), cudaMemcpyHostToDevice, e->stream));
        CK(cudaMemsetAsync(e->d_fd.p, 0, 2 * np * nf * sizeof(double), e->stream));
        CK(cudaMemsetAsync(e->d_fd_count.p, 0, sizeof(int), e->stream));
        e->fd.nfreq = (int)nf;
        e->fd.freq = e->d_freq.p;
        e->fd.acc = e->d_fd.p;
        e->fd.dual = e->d_fd_dual.p;
        e->fd.dT = e->dT;
        e->fd.scale = 2.0 * e->dT * (double)e->fd_interval;
        e->fd.count = e->d_fd_count.p;
    }
    e->probes_uploaded = true;
    return FDTD_OK;
}

int build_chunk_graph(fdtd_engine_s* e) {
    if (e->chunk) return FDTD_OK;
    cudaGraph_t graph = nullptr;
    CK(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
    int rc = FDTD_OK;
    const uint64_t saved = e->last_launches;
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

int start(fdtd_engine_s* e) {
    int rc;
    if (!e->started) {
        if ((rc = upload_probes(e))) return rc;
        e->started = true;
        if (e->interval && e->use_graphs && (rc = build_chunk_graph(e))) return rc;
    }
    if (e->need_initial_sample) {
        e->need_initial_sample = false;
        if (e->interval) {  // sample at ts = 0 (RunFDTD's PA->Process() before the loop)
            if ((rc = launch_advance(e, 0, true, e->energy_on_probe))) return rc;
        }
        if ((rc = launch_fd(e, 0))) return rc;  // 0 % FD_interval == 0
    }
    return FDTD_OK;
}

int decode_error(int err) {
    if (err & 4) {
        set_error("a bounded device wait gave up: a TMA copy did not complete in time");
        return FDTD_ERR_TIMEOUT;
    }
    if (err & 1) {
        set_error("probe sample ring overflow: raise max_timesteps");
        return FDTD_ERR_STATE;
    }
    if (err & 2) {
        set_error("energy reduction is not finite (NaN/Inf in the fields)");
        return FDTD_ERR_NONFINITE;
    }
    return FDTD_OK;
}

// Reads the control words back: numTS (which stops advancing once a device
// end criterion is met) and the error word.
int check_error_word(fdtd_engine_s* e) {
    int ctl[4] = {0, 0, 0, 0};
    CK(cudaMemcpyAsync(ctl, e->ctl.p, sizeof(ctl), cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    e->ts = (uint32_t)ctl[0];
    e->done = ctl[3] != 0;
    return decode_error(ctl[2]);
}
// --------------------------------------------------------------- TMA maps
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

int index_map(CUtensorMap* m, void* base, const fdtd_engine_s* e, bool idx16, uint32_t box_z = 32,
              uint32_t box_y = TMA_TY) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc) {
        set_error("cuTensorMapEncodeTiled is not available from the driver");
        return FDTD_ERR_CUDA;
    }
    const cuuint64_t ib = idx16 ? 2 : 4;
    cuuint64_t dims[3] = {e->N[2], e->N[1], e->N[0]};
    cuuint64_t strides[2] = {(cuuint64_t)e->Nzp * ib, (cuuint64_t)e->N[1] * e->Nzp * ib};
    cuuint32_t box[3] = {box_z, box_y, 1};
    cuuint32_t es[3] = {1, 1, 1};
    CUresult r = enc(m, idx16 ? CU_TENSOR_MAP_DATA_TYPE_UINT16 : CU_TENSOR_MAP_DATA_TYPE_UINT32, 3, base, dims, strides,
                     box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled (index) failed: " + std::to_string((int)r));
        return FDTD_ERR_CUDA;
    }
    return FDTD_OK;
}

// tensor maps of the fused kernel (boxes: see kernels_fused.cuh)
int make_fused_maps(fdtd_engine_s* e) {
    int rc;
    FusedMaps& m = e->fmaps;
    float* Vb[2] = {e->V.p, e->V2.p};
    float* Ib[2] = {e->I.p, e->I2.p};
    float* Fb[2] = {e->FV.p, e->FV2.p};
    for (int p = 0; p < 2; ++p) {
        if ((rc = field_map(&m.I_halo[p], Ib[p], e, FU_IW, FU_IH)) ||
            (rc = field_map(&m.V_ext[p], Vb[p], e, FU_VW, FU_EH)))
            return rc;
        if (Fb[p] && (rc = field_map(&m.FV_ext[p], Fb[p], e, FU_VW, FU_EH))) return rc;
    }
    if (e->FI.p && (rc = field_map(&m.FI_own, e->FI.p, e, 32, FU_TY))) return rc;
    if ((rc = index_map(&m.idxE_ext, e->E.idx.p, e, e->E.idx16, FU_XW, FU_EH)) ||
        (rc = index_map(&m.idxH_own, e->H.idx.p, e, e->H.idx16, 32, FU_TY)))
        return rc;
    return FDTD_OK;
}

template <typename IE, typename IH>
cudaError_t fused_attr_one(int bytes) {
    const cudaFuncAttribute a = cudaFuncAttributeMaxDynamicSharedMemorySize;
    cudaError_t r[4] = {cudaFuncSetAttribute(k_step_fused<IE, IH, 0, false>, a, bytes),
                        cudaFuncSetAttribute(k_step_fused<IE, IH, 0, true>, a, bytes),
                        cudaFuncSetAttribute(k_step_fused<IE, IH, FEAT_UPML, false>, a, bytes),
                        cudaFuncSetAttribute(k_step_fused<IE, IH, FEAT_UPML, true>, a, bytes)};
    for (cudaError_t x : r)
        if (x != cudaSuccess) return x;
    return cudaSuccess;
}

int set_fused_attrs(int bytes) {
    cudaError_t r = cudaSuccess, t;
    if ((t = fused_attr_one<uint16_t, uint16_t>(bytes)) != cudaSuccess) r = t;
    if ((t = fused_attr_one<uint16_t, uint32_t>(bytes)) != cudaSuccess) r = t;
    if ((t = fused_attr_one<uint32_t, uint16_t>(bytes)) != cudaSuccess) r = t;
    if ((t = fused_attr_one<uint32_t, uint32_t>(bytes)) != cudaSuccess) r = t;
    if (r != cudaSuccess) {
        set_error(std::string("cudaFuncSetAttribute(MaxDynamicSharedMemorySize, fused): ") + cudaGetErrorString(r));
        return FDTD_ERR_CUDA;
    }
    return FDTD_OK;
}

// the two-pass kernels' tensor maps for tiles of `rows` y rows
int make_tma_maps(const fdtd_engine_s* e, TmaMaps* m, uint32_t rows) {
    int rc;
    if ((rc = field_map(&m->I_halo, e->I.p, e, 36, rows + 1)) || (rc = field_map(&m->I_own, e->I.p, e, 32, rows)) ||
        (rc = field_map(&m->V_halo, e->V.p, e, 36, rows + 1)) || (rc = field_map(&m->V_own, e->V.p, e, 32, rows)) ||
        (rc = index_map(&m->idxE, e->E.idx.p, e, e->E.idx16, 32, rows)) ||
        (rc = index_map(&m->idxH, e->H.idx.p, e, e->H.idx16, 32, rows)))
        return rc;
    if (e->FV.p && ((rc = field_map(&m->FV_own, e->FV.p, e, 32, rows)) ||
                    (rc = field_map(&m->FI_own, e->FI.p, e, 32, rows))))
        return rc;
    if (e->AV.p && (rc = field_map(&m->AV_own, e->AV.p, e, 32, rows))) return rc;
    if (e->LV.p && (rc = field_map(&m->LV_own, e->LV.p, e, 32, rows))) return rc;
    return FDTD_OK;
}

int make_maps(fdtd_engine_s* e) { return make_tma_maps(e, &e->maps, (uint32_t)e->tma_ty); }

int set_smem_attrs(int bytes) {
    cudaError_t r = cudaSuccess, t;
#define WIPEMS_ATTR(I, F)                                                 \
    if ((t = smem_attr_one<I, F, false>(bytes)) != cudaSuccess) r = t;    \
    if ((t = smem_attr_one<I, F, true>(bytes)) != cudaSuccess) r = t;
    WIPEMS_ATTR(uint16_t, 0) WIPEMS_ATTR(uint16_t, 1) WIPEMS_ATTR(uint16_t, 2) WIPEMS_ATTR(uint16_t, 3)
    WIPEMS_ATTR(uint32_t, 0) WIPEMS_ATTR(uint32_t, 1) WIPEMS_ATTR(uint32_t, 2) WIPEMS_ATTR(uint32_t, 3)
#undef WIPEMS_ATTR
    if ((t = smem_attrs_adex(bytes)) != cudaSuccess) r = t;
    if (r != cudaSuccess) {
        set_error(std::string("cudaFuncSetAttribute(MaxDynamicSharedMemorySize): ") + cudaGetErrorString(r));
        return FDTD_ERR_CUDA;
    }
    return FDTD_OK;
}

// ----------------------------------------------------------- engine state
// Engine::Init state: all fields and extension states zero, numTS = 0,
// no recorded samples (the ts = 0 sample is taken again on the next iterate).
int reset_state(fdtd_engine_s* e) {
    cudaStream_t s = e->stream;
    const size_t F = 3 * (size_t)e->comp * sizeof(float);
    for (DevBuf<float>* b : {&e->V, &e->I, &e->FV, &e->FI, &e->AV, &e->LV, &e->AI, &e->LI, &e->V2, &e->I2, &e->FV2})
        if (b->p) CK(cudaMemsetAsync(b->p, 0, F, s));
    for (DevBuf<float>* b : {&e->AVx, &e->LVx, &e->AIx, &e->LIx})
        if (b->p) CK(cudaMemsetAsync(b->p, 0, b->n * sizeof(float), s));
    CK(cudaMemsetAsync(e->ctl.p, 0, 4 * sizeof(int), s));
    if (e->d_fd.p) CK(cudaMemsetAsync(e->d_fd.p, 0, e->d_fd.n * sizeof(double), s));
    if (e->mur_buf.p) CK(cudaMemsetAsync(e->mur_buf.p, 0, e->mur_buf.n * sizeof(float), s));
    if (e->rlc_state.p) CK(cudaMemsetAsync(e->rlc_state.p, 0, e->rlc_state.n * sizeof(float), s));
    if (e->d_fd_count.p) CK(cudaMemsetAsync(e->d_fd_count.p, 0, sizeof(int), s));
    CK(cudaMemsetAsync(e->d_eacc.p, 0, 4 * sizeof(double), s));
    // the ts = 0 sample reads the plane sums of the zero fields
    CK(cudaMemsetAsync(e->eplane.p, 0, e->eplane.n * sizeof(double2), s));
    e->ts = 0;
    e->done = false;
    e->need_initial_sample = true;
    return FDTD_OK;
}

int upload_half(fdtd_engine_s* e, const HalfTables& T, DevHalfBufs& B, DevHalf& D) {
    int rc;
    uint64_t& tot = e->device_bytes;
    B.idx16 = T.idx16;
    cudaStream_t st = e->stream;
    if ((rc = B.idx.alloc(T.idx_bytes, tot, st)) || (rc = B.main.alloc(T.main.size(), tot, st)) ||
        (rc = B.exc.alloc(std::max<size_t>(4, T.exc.size()), tot, st)) ||
        (rc = B.upml.alloc(T.upml.size(), tot, st)) || (rc = B.ade.alloc(T.ade.size(), tot, st)) ||
        (rc = B.adex.alloc(T.adex.size(), tot, st)))
        return rc;
    auto h2d = [&](void* dst, const void* src, size_t bytes) -> cudaError_t {
        return bytes ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, e->stream) : cudaSuccess;
    };
    CK(h2d(B.idx.p, T.idx, T.idx_bytes));
    CK(h2d(B.main.p, T.main.data(), T.main.size() * sizeof(float)));
    CK(h2d(B.exc.p, T.exc.data(), T.exc.size() * sizeof(float)));
    CK(h2d(B.upml.p, T.upml.data(), T.upml.size() * sizeof(float)));
    CK(h2d(B.ade.p, T.ade.data(), T.ade.size() * sizeof(float)));
    CK(h2d(B.adex.p, T.adex.data(), T.adex.size() * sizeof(float)));
    D.idx = B.idx.p;
    D.main = reinterpret_cast<const float4*>(B.main.p);
    D.upml = reinterpret_cast<const float4*>(B.upml.p);
    D.ade = reinterpret_cast<const float4*>(B.ade.p);
    D.exc = reinterpret_cast<const float4*>(B.exc.p);
    D.adex = reinterpret_cast<const float4*>(B.adex.p);
    D.ntup = (int)T.num_tuples;
    return FDTD_OK;
}

int upload_engine(const fdtd_cop_s* c, const fdtd_engine_opts* opts, fdtd_engine_s* e) {
    for (int a = 0; a < 3; ++a) {
        e->N[a] = c->N[a];
        e->N0[a] = c->N0[a];
    }
    e->rot = c->rot;
    e->dT = c->dT;
    e->device = opts ? opts->device : 0;
    CK(cudaSetDevice(e->device));
    CK(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking));
    {  // keep freed pool memory in this process for the next engine (no return to the driver)
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, e->device) == cudaSuccess) {
            uint64_t keep = UINT64_MAX;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
    }
    CK(cudaEventCreate(&e->ev0));
    CK(cudaEventCreate(&e->ev1));
    e->TY = (opts && opts->tile_y > 0) ? opts->tile_y : 8;
    if (e->TY > 8 || e->TY < 1) {
        set_error("tile_y must be 1..8");
        return FDTD_ERR_ARG;
    }
    e->XC = (opts && opts->x_chunk > 0) ? opts->x_chunk : 0;  // 0: auto_x_chunk below
    e->interval = opts ? opts->probe_interval : 0;
    e->energy_on_probe = opts ? opts->energy_on_probe != 0 : true;
    e->use_graphs = opts ? opts->use_graphs != 0 : true;
    const int kern = opts ? opts->kernel : 0;
    if (kern < 0 || kern > 3) {
        set_error("kernel must be 0 (auto), 1 (direct), 2 (fused) or 3 (two-pass TMA)");
        return FDTD_ERR_ARG;
    }
    e->use_tma = kern != 1;
    e->fused = kern == 2;
    // the two-pass TMA kernels come in 4- and 8-row tiles (4 by default)
    e->tma_ty = (opts && opts->tile_y > 0) ? opts->tile_y : TMA_TY;
    if (e->use_tma && !e->fused && e->tma_ty != 4 && e->tma_ty != 8) {
        set_error("the TMA kernels take tile_y 4 or 8 (0 = 4)");
        return FDTD_ERR_ARG;
    }
    e->stages = (opts && opts->stages > 0) ? opts->stages : 3;
    if (e->stages < 3 || e->stages > TMA_MAX_STAGES) {
        set_error("stages must be 3..8");
        return FDTD_ERR_ARG;
    }
    const uint32_t maxts = (opts && opts->max_timesteps) ? opts->max_timesteps : 100000;
    e->cap = (e->interval ? maxts / e->interval : 0) + 2;
    e->end_crit = opts ? opts->end_crit : 0.0;
    e->stop_ts = maxts;
    if (e->end_crit < 0 || (e->end_crit > 0 && (!e->interval || !e->energy_on_probe))) {
        set_error("end_crit needs probe_interval > 0 and energy_on_probe (the energy is checked on sample steps)");
        return FDTD_ERR_ARG;
    }
    e->num_tuples_e = c->E.num_tuples;
    e->num_tuples_h = c->H.num_tuples;
    e->upml_nodes = c->upml_nodes;
    e->ade_nodes = c->ade_nodes;
    e->Nzp = c->Nzp;
    if (e->XC == 0) {
        int sms = 0;
        CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, e->device));
        // about 1280 resident threads per SM (5 blocks of 32 x 8, 10 of 32 x 4)
        e->XC = auto_x_chunk({e->N}, (uint64_t)(1280 / (32 * e->tma_ty)) * (uint64_t)sms);
    }
    e->comp = c->comp;
    e->geo_on = c->geo;
    const bool any_upml = c->E.any_upml || c->H.any_upml;
    const bool any_adex = c->E.adex_orders || c->H.adex_orders;
    const bool any_ade = c->E.any_ade || c->H.any_ade || any_adex;
    e->feat = (any_upml ? FEAT_UPML : 0) | (any_ade ? FEAT_ADE : 0) | (any_adex ? FEAT_ADEX : 0);
    // each half-step kernel carries only the extensions its own tuples use
    // (a scene with electric dispersion only runs the current kernel
    // without the ADE terms: fewer registers, more resident blocks)
    auto half_feat = [&](const HalfTables& T) {
        return (any_upml ? FEAT_UPML : 0) | ((T.any_ade || T.adex_orders) ? FEAT_ADE : 0) |
               (T.adex_orders ? FEAT_ADEX : 0);
    };
    e->feat_e = half_feat(c->E);
    e->feat_h = half_feat(c->H);
    if (e->fused && (any_ade || c->geo)) {
        set_error("the fused single-pass kernel does not cover Lorentz/Drude nodes or factorized geometry "
                  "(use the two-pass TMA kernels)");
        return FDTD_ERR_UNSUPPORTED;
    }

    int rc;
    uint64_t& tot = e->device_bytes;
    const size_t F = 3 * (size_t)e->comp;
    if ((rc = e->V.alloc(F, tot, e->stream)) || (rc = e->I.alloc(F, tot, e->stream))) return rc;
    if (any_upml && ((rc = e->FV.alloc(F, tot, e->stream)) || (rc = e->FI.alloc(F, tot, e->stream)))) return rc;
    if (e->fused && ((rc = e->V2.alloc(F, tot, e->stream)) || (rc = e->I2.alloc(F, tot, e->stream)))) return rc;
    if (e->fused && any_upml && (rc = e->FV2.alloc(F, tot, e->stream))) return rc;
    if (c->E.any_ade && (rc = e->AV.alloc(F, tot, e->stream))) return rc;
    if (c->E.any_lor && (rc = e->LV.alloc(F, tot, e->stream))) return rc;
    if (c->H.any_ade && (rc = e->AI.alloc(F, tot, e->stream))) return rc;
    if (c->H.any_lor && (rc = e->LI.alloc(F, tot, e->stream))) return rc;
    if (c->E.adex_orders && (rc = e->AVx.alloc(c->E.adex_orders * F, tot, e->stream))) return rc;
    if (c->E.any_lorx && (rc = e->LVx.alloc(c->E.adex_orders * F, tot, e->stream))) return rc;
    if (c->H.adex_orders && (rc = e->AIx.alloc(c->H.adex_orders * F, tot, e->stream))) return rc;
    if (c->H.any_lorx && (rc = e->LIx.alloc(c->H.adex_orders * F, tot, e->stream))) return rc;
    if ((rc = e->sigV.alloc(std::max<uint32_t>(1, c->sig_len), tot, e->stream)) ||
        (rc = e->sigC.alloc(std::max<uint32_t>(1, c->sig_len), tot, e->stream)))
        return rc;
    if ((rc = e->ctl.alloc(4, tot, e->stream)) || (rc = e->d_eacc.alloc(4, tot, e->stream)) ||
        (rc = e->d_energy_tmp.alloc(2, tot, e->stream)))
        return rc;
    // energy segments: one float pair per (x < Nx-1, y < Ny-1, 32-node z tile)
    const int nzt = ((int)e->N[2] - 1 + 31) / 32;
    if ((rc = e->eseg.alloc((size_t)(e->N[0] - 1) * (e->N[1] - 1) * (size_t)nzt, tot, e->stream)) ||
        (rc = e->eplane.alloc(e->N[0] - 1, tot, e->stream)))
        return rc;
    DevGrid& g = e->g;
    if ((rc = upload_half(e, c->E, e->E, g.e)) || (rc = upload_half(e, c->H, e->H, g.h))) return rc;
    if (c->geo) {
        if ((rc = e->geo.alloc(c->geom.size(), tot, e->stream))) return rc;
        CK(cudaMemcpyAsync(e->geo.p, c->geom.data(), c->geom.size() * sizeof(float), cudaMemcpyHostToDevice,
                           e->stream));
    }
    if (c->sig_len) {
        CK(cudaMemcpyAsync(e->sigV.p, c->sigV.data(), c->sig_len * sizeof(float), cudaMemcpyHostToDevice, e->stream));
        CK(cudaMemcpyAsync(e->sigC.p, c->sigC.data(), c->sig_len * sizeof(float), cudaMemcpyHostToDevice, e->stream));
    } else {
        CK(cudaMemsetAsync(e->sigV.p, 0, sizeof(float), e->stream));
        CK(cudaMemsetAsync(e->sigC.p, 0, sizeof(float), e->stream));
    }
    if (!c->mur.empty()) {
        if (e->fused) {
            set_error("the fused single-pass kernel does not cover Mur boundaries (use the two-pass kernels)");
            return FDTD_ERR_UNSUPPORTED;
        }
        size_t tot_n = 0;
        for (const MurFace& M : c->mur) tot_n += (size_t)M.n[0] * M.n[1];
        if ((rc = e->mur_coef.alloc(2 * tot_n, tot, e->stream)) || (rc = e->mur_buf.alloc(2 * tot_n, tot, e->stream)))
            return rc;
        CK(cudaMemsetAsync(e->mur_buf.p, 0, 2 * tot_n * sizeof(float), e->stream));
        std::vector<float> hc(2 * tot_n);
        size_t off = 0;
        e->mur.nface = 0;
        for (const MurFace& M : c->mur) {
            const size_t n = (size_t)M.n[0] * M.n[1];
            std::copy(M.cp.begin(), M.cp.end(), hc.begin() + 2 * off);
            std::copy(M.cpp.begin(), M.cpp.end(), hc.begin() + 2 * off + n);
            MurDev& F = e->mur.f[e->mur.nface++];
            F.ny = M.ny;
            F.line = (int)M.line;
            F.shift = (int)M.shift;
            F.n0 = (int)M.n[0];
            F.n1 = (int)M.n[1];
            F.start_ts = (int)M.start_ts;
            F.cp = e->mur_coef.p + 2 * off;
            F.cpp = e->mur_coef.p + 2 * off + n;
            F.bp = e->mur_buf.p + 2 * off;
            F.bpp = e->mur_buf.p + 2 * off + n;
            F.offset = (uint32_t)off;
            off += n;
        }
        e->mur.total = (uint32_t)tot_n;
        e->mur.idx16 = c->E.idx16 ? 1 : 0;
        for (int a = 0; a < 3; ++a) e->mur.trim[a] = c->trim_e[a] ? 1 : 0;
        CK(cudaMemcpyAsync(e->mur_coef.p, hc.data(), hc.size() * sizeof(float), cudaMemcpyHostToDevice, e->stream));
    }
    if (c->rlc.size()) {
        if (e->fused) {
            set_error("the fused single-pass kernel does not cover lumped RLC elements (use the two-pass kernels)");
            return FDTD_ERR_UNSUPPORTED;
        }
        const size_t n = c->rlc.size();
        if ((rc = e->rlc_coef.alloc(9 * n, tot, e->stream)) || (rc = e->rlc_state.alloc(7 * n, tot, e->stream)) ||
            (rc = e->rlc_off.alloc(n, tot, e->stream)))
            return rc;
        std::vector<float> hc(9 * n);
        std::vector<long long> ho(n);
        const RlcList& r = c->rlc;
        const std::vector<float>* cols[9] = {&r.ilv, &r.i2v, &r.vv2, &r.vj1, &r.vj2, &r.vvd, &r.ib0, &r.b1, &r.b2};
        for (int q = 0; q < 9; ++q) std::copy(cols[q]->begin(), cols[q]->end(), hc.begin() + q * n);
        for (size_t k = 0; k < n; ++k)
            ho[k] = (long long)r.dir[k] * e->comp + ((long long)r.pos[0][k] * e->N[1] + r.pos[1][k]) * e->Nzp +
                    r.pos[2][k];
        CK(cudaMemcpyAsync(e->rlc_coef.p, hc.data(), hc.size() * sizeof(float), cudaMemcpyHostToDevice, e->stream));
        CK(cudaMemcpyAsync(e->rlc_off.p, ho.data(), n * sizeof(long long), cudaMemcpyHostToDevice, e->stream));
        CK(cudaMemsetAsync(e->rlc_state.p, 0, 7 * n * sizeof(float), e->stream));
        CK(cudaStreamSynchronize(e->stream));  // the host staging vectors end here
        e->rlc.count = (uint32_t)n;
        e->rlc.off = e->rlc_off.p;
        e->rlc.coef = e->rlc_coef.p;
        e->rlc.state = e->rlc_state.p;
    }
    g.Nx = (int)e->N[0];
    g.Ny = (int)e->N[1];
    g.Nz = (int)e->N[2];
    g.Nzp = e->Nzp;
    g.sx = (long long)e->N[1] * e->Nzp;
    g.comp = e->comp;
    g.V = e->V.p;
    g.I = e->I.p;
    g.V2 = e->V2.p;
    g.I2 = e->I2.p;
    g.FV2 = e->FV2.p;
    g.FV = e->FV.p;
    g.FI = e->FI.p;
    g.AV = e->AV.p;
    g.LV = e->LV.p;
    if (!c->edges.empty()) {
        e->h_edges = c->edges;
        if ((rc = e->edges.alloc(c->edges.size(), tot, e->stream))) return rc;
        CK(cudaMemcpy(e->edges.p, c->edges.data(), c->edges.size() * sizeof(double), cudaMemcpyHostToDevice));
    }
    if (c->E.any_ade) {  // which voltage-kernel tile planes hold Lorentz/Drude nodes
        const int ZT = ((int)e->N[2] + 31) / 32, YT = ((int)e->N[1] + TMA_TY - 1) / TMA_TY;
        std::vector<uint8_t> tf(c->E.num_tuples);
        for (uint32_t k = 0; k < c->E.num_tuples; ++k) {
            uint32_t f;
            std::memcpy(&f, &c->E.main[(size_t)k * TAB_MAIN * 4 + 6], 4);
            tf[k] = (uint8_t)(((f & TF_ADE) ? 1u : 0u) | ((f & TF_LOR) ? 2u : 0u));
        }
        std::vector<uint8_t> h((size_t)e->N[0] * YT * ZT, 0);
        for (uint32_t x = 0; x < e->N[0]; ++x)
            for (uint32_t y = 0; y < e->N[1]; ++y) {
                const size_t row = ((size_t)x * e->N[1] + y) * (size_t)e->Nzp;
                uint8_t* hf = &h[((size_t)x * YT + y / TMA_TY) * ZT];
                for (uint32_t z = 0; z < e->N[2]; ++z) {
                    const uint32_t t = c->E.idx16 ? reinterpret_cast<const uint16_t*>(c->E.idx)[row + z]
                                                  : reinterpret_cast<const uint32_t*>(c->E.idx)[row + z];
                    hf[z / 32] |= tf[t];
                }
            }
        if ((rc = e->ade_tile.alloc(h.size(), tot, e->stream))) return rc;
        CK(cudaMemcpy(e->ade_tile.p, h.data(), h.size(), cudaMemcpyHostToDevice));
        g.ade_tile = e->ade_tile.p;
    } else {
        g.ade_tile = nullptr;
    }
    g.AI = e->AI.p;
    g.LI = e->LI.p;
    g.AVx = e->AVx.p;
    g.LVx = e->LVx.p;
    g.AIx = e->AIx.p;
    g.LIx = e->LIx.p;
    g.geo = e->geo.p;
    g.geo_stride = (int)(e->N[0] + e->N[1] + e->N[2]);
    g.sigV = e->sigV.p;
    g.sigC = e->sigC.p;
    g.sig_len = (int)c->sig_len;
    g.sig_period = (int)c->sig_period;
    g.d_ts = e->p_ts();
    g.d_done = e->p_done();
    g.d_eacc = e->d_eacc.p;
    g.eseg = e->eseg.p;
    g.eplane = e->eplane.p;
    g.nzt = ((int)e->N[2] - 1 + 31) / 32;
    e->smem_direct = 2 * 3 * (size_t)(e->TY + 1) * 33 * sizeof(float);
    for (int a = 0; a < 3; ++a) {
        e->ti.lo[a] = c->inner_lo[a];
        e->ti.hi[a] = c->inner_hi[a];
        e->ti.ne[a] = (int)e->N[a] - (c->trim_e[a] ? 1 : 0);
    }
    e->ti.d_err = e->p_err();
    if (e->fused) {
        if ((rc = make_fused_maps(e))) return rc;
        const size_t need = FusedLayout<uint32_t, uint32_t, true>::smem(e->stages);
        if (need > 48 * 1024 && (rc = set_fused_attrs((int)need))) return rc;
    } else if (e->use_tma) {
        if ((rc = make_maps(e))) return rc;
        const size_t need = e->tma_ty == 8
                                ? ((e->feat & FEAT_UPML) ? StageLayout<uint32_t, true, true, 8>::smem(e->stages)
                                                         : StageLayout<uint32_t, false, true, 8>::smem(e->stages))
                                : ((e->feat & FEAT_UPML) ? StageLayout<uint32_t, true, true>::smem(e->stages)
                                                         : StageLayout<uint32_t, false, true>::smem(e->stages));
        if (need > 48 * 1024 && (rc = set_smem_attrs((int)need))) return rc;
    }
    return reset_state(e);
}

// Probe entries for ProcessVoltage (Engine_Interface_FDTD::CalcVoltageIntegral,
// engine_interface_fdtd.cpp:200-226) and ProcessCurrent::CalcIntegral
// (processcurrent.cpp:93-168), as (component, node, sign) lists.
// The entries of an integral probe, built in the operator's axes in the
// reference's walk order and mapped to device nodes one by one (so the
// device sums run in the reference's order whatever the device axes).
int probe_entries(const fdtd_engine_s* e, const fdtd_probe_desc* p, std::vector<ProbeEntry>& out) {
    auto add = [&](int field, int comp, uint32_t x, uint32_t y, uint32_t z, int sign) -> int {
        if (x >= e->N0[0] || y >= e->N0[1] || z >= e->N0[2]) {
            set_error("probe position outside the grid");
            return FDTD_ERR_ARG;
        }
        ProbeEntry pe;
        const uint32_t o[3] = {x, y, z};
        pe.off = e->dev_offset(o);
        pe.comp = (int8_t)e->dev_comp(comp);
        pe.sign = (int8_t)sign;
        pe.field = (int8_t)field;
        std::memset(pe.pad, 0, sizeof(pe.pad));
        out.push_back(pe);
        return FDTD_OK;
    };
    if (!p->enabled) return FDTD_OK;
    const uint32_t* start = p->start;
    const uint32_t* stop = p->stop;
    if (p->type == 0) {
        const int dims = (start[0] != stop[0]) + (start[1] != stop[1]) + (start[2] != stop[2]);
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

int engine_start(fdtd_engine_s* e) { return start(e); }
int engine_tma_maps(const fdtd_engine_s* e, TmaMaps* out, uint32_t rows) { return make_tma_maps(e, out, rows); }
int engine_check_errors(fdtd_engine_s* e) { return check_error_word(e); }
int engine_decode_error(int err) { return decode_error(err); }
int engine_auto_x_chunk(const uint32_t N[3], int device, unsigned share) {
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || sms <= 0) return 0;
    const uint64_t resident = (uint64_t)(1280 / (32 * TMA_TY)) * (uint64_t)sms / (share > 0 ? share : 1);
    return auto_x_chunk({N}, resident > 0 ? resident : 1);
}

}  // namespace wipems

// ===================================================================== C ABI
extern "C" {

int fdtd_engine_create_compressed(fdtd_cop_t cop, const fdtd_engine_opts* opts, fdtd_engine_t* out) {
    if (!cop || !out) {
        set_error("fdtd_engine_create_compressed: null argument");
        return FDTD_ERR_ARG;
    }
    fdtd_engine_s* e = new (std::nothrow) fdtd_engine_s();
    if (!e) return FDTD_ERR_NOMEM;
    int rc;
    try {
        rc = upload_engine(cop, opts, e);
    } catch (const std::bad_alloc&) {
        set_error("fdtd_engine_create: host allocation failed");
        rc = FDTD_ERR_NOMEM;
    }
    if (rc == FDTD_OK) {
        const cudaError_t ce = cudaStreamSynchronize(e->stream);
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
    if (p->type == 2 || p->type == 3) {  // field probe: three columns, one entry each
        const bool h = p->type == 3;
        for (int a = 0; a < 3; ++a)
            if (p->start[a] >= e->N0[a]) {
                set_error("fdtd_engine_add_probe: field probe outside the grid");
                return FDTD_ERR_ARG;
            }
        if (p->enabled && e->h_edges.empty()) {
            set_error("fdtd_engine_add_probe: field probes need the mesh lines in the operator description");
            return FDTD_ERR_STATE;
        }
        if (slot) *slot = (uint32_t)e->h_weight.size();
        const size_t ntot = (size_t)e->N[0] + e->N[1] + e->N[2];
        const size_t eoff[3] = {0, e->N[0], (size_t)e->N[0] + e->N[1]};  // edge arrays in device axes
        for (int n = 0; n < 3; ++n) {  // columns in the operator's component order
            double dv = -1.0;  // disabled probe or zero edge length: the column reads 0
            if (p->enabled) {
                ProbeEntry pe{};
                pe.off = e->dev_offset(p->start);
                pe.comp = (int8_t)e->dev_comp(n);
                pe.sign = 1;
                pe.field = (int8_t)(h ? 1 : 0);
                e->h_entries.push_back(pe);
                const double len = e->h_edges[(h ? ntot : 0) + eoff[e->dev_comp(n)] + p->start[n]];
                if (len != 0.0) dv = len;
            }
            e->h_first.push_back((int)e->h_entries.size());
            e->h_weight.push_back(p->weight);
            e->h_div.push_back(dv);
            e->h_dual.push_back(h ? 1 : 0);
        }
        return FDTD_OK;
    }
    std::vector<ProbeEntry> ent;
    const int rc = probe_entries(e, p, ent);
    if (rc) return rc;
    e->h_entries.insert(e->h_entries.end(), ent.begin(), ent.end());
    e->h_first.push_back((int)e->h_entries.size());
    e->h_weight.push_back(p->weight);
    e->h_div.push_back(0.0);
    e->h_dual.push_back(p->type == 1 ? 1 : 0);
    if (slot) *slot = (uint32_t)(e->h_weight.size() - 1);
    return FDTD_OK;
}

int fdtd_engine_iterate(fdtd_engine_t e, uint32_t n) {
    const int rc = fdtd_engine_iterate_async(e, n);
    if (rc) return rc;
    return fdtd_engine_wait(e);
}

int fdtd_engine_wait(fdtd_engine_t e) {
    if (!e) return FDTD_ERR_ARG;
    if (!e->pending) return FDTD_OK;
    CK(cudaSetDevice(e->device));
    e->pending = false;
    CK(cudaEventSynchronize(e->ev1));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, e->ev0, e->ev1));
    e->last_ms = ms;
    return check_error_word(e);
}

int fdtd_engine_iterate_async(fdtd_engine_t e, uint32_t n) {
    if (!e) return FDTD_ERR_ARG;
    if (e->pending) {
        set_error("fdtd_engine_iterate_async: the previous asynchronous iterate was not waited for");
        return FDTD_ERR_STATE;
    }
    if (e->end_crit > 0) {  // a stopped job stays stopped; never step past the timestep cap
        if (e->done || e->ts >= e->stop_ts) n = 0;
        else n = std::min(n, e->stop_ts - e->ts);
    }
    CK(cudaSetDevice(e->device));
    e->last_launches = 0;
    int rc;
    CK(cudaEventRecord(e->ev0, e->stream));
    if ((rc = start(e))) return rc;
    const bool fd_on = e->fd_interval && !e->h_freq.empty() && e->ps.nprobe;
    uint32_t left = n;
    while (left > 0) {
        // steps to the next frequency-domain step (a chunk graph may end on
        // it, not pass it)
        const uint32_t to_fd = fd_on ? e->fd_interval - (e->ts % e->fd_interval) : ~0u;
        if (e->interval && e->use_graphs && e->chunk && (e->ts % e->interval) == 0 && left >= e->interval &&
            to_fd >= e->interval) {
            CK(cudaGraphLaunch(e->chunk, e->stream));
            e->last_launches += (e->fused ? 1 : 2) * (uint64_t)e->interval + 1 + (e->energy_on_probe ? 1 : 0);
            e->ts += e->interval;
            left -= e->interval;
            if (to_fd == e->interval && (rc = launch_fd(e, e->ts))) return rc;
            continue;
        }
        const bool sample = e->interval && ((e->ts + 1) % e->interval) == 0;
        if ((rc = launch_step(e, 0, sample && e->energy_on_probe))) return rc;
        if ((rc = launch_advance(e, 1, sample, e->energy_on_probe))) return rc;
        e->ts += 1;
        left -= 1;
        if (fd_on && (e->ts % e->fd_interval) == 0 && (rc = launch_fd(e, e->ts))) return rc;
    }
    CK(cudaEventRecord(e->ev1, e->stream));
    e->pending = true;
    return FDTD_OK;
}

int fdtd_engine_set_fd(fdtd_engine_t e, const double* freqs, uint32_t nfreq, uint32_t fd_interval) {
    if (!e || (nfreq && !freqs)) return FDTD_ERR_ARG;
    if (e->started) {
        set_error("fdtd_engine_set_fd: frequencies must be set before the first iterate");
        return FDTD_ERR_STATE;
    }
    if (nfreq && fd_interval == 0) {
        set_error("fdtd_engine_set_fd: fd_interval must be > 0");
        return FDTD_ERR_ARG;
    }
    e->h_freq.assign(freqs, freqs + nfreq);
    e->fd_interval = nfreq ? fd_interval : 0;
    return FDTD_OK;
}

int fdtd_engine_read_fd(fdtd_engine_t e, double* re_im, uint32_t* samples) {
    if (!e) return FDTD_ERR_ARG;
    if (e->pending) {
        set_error("fdtd_engine_read_fd: wait for the asynchronous iterate first");
        return FDTD_ERR_STATE;
    }
    CK(cudaSetDevice(e->device));
    int cnt = 0;
    if (e->d_fd.p) {
        if (re_im)
            CK(cudaMemcpyAsync(re_im, e->d_fd.p, e->d_fd.n * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
        CK(cudaMemcpyAsync(&cnt, e->d_fd_count.p, sizeof(int), cudaMemcpyDeviceToHost, e->stream));
        CK(cudaStreamSynchronize(e->stream));
    }
    if (samples) *samples = (uint32_t)cnt;
    return FDTD_OK;
}

// ------------------------------------------------------------ checkpoints
// Blob: a header, then every piece of device state as (element count, raw
// bytes) in a fixed order; restore checks each count against the engine.
namespace {
struct CkptHeader {
    char magic[8];
    uint32_t version;
    uint32_t N[3];
    int32_t Nzp;
    uint32_t nprobe, row_doubles, nfreq, nmur;
    uint32_t ts, done, nsamp;
    int32_t frame;  // bit 0: fused single-pass kernel; bits 1-2: the device axis rotation
    uint32_t nrlc;
};

struct CkptPart {
    void* p;
    size_t bytes;
};

std::vector<CkptPart> ckpt_parts(fdtd_engine_s* e, uint32_t nsamp) {
    std::vector<CkptPart> v;
    auto add = [&](void* p, size_t bytes) { v.push_back(CkptPart{p, p ? bytes : 0}); };
    const size_t F = 3 * (size_t)e->comp * sizeof(float);
    add(e->ctl.p, 4 * sizeof(int));
    add(e->d_eacc.p, 4 * sizeof(double));
    for (DevBuf<float>* b : {&e->V, &e->I, &e->FV, &e->FI, &e->AV, &e->LV, &e->AI, &e->LI, &e->V2, &e->I2, &e->FV2})
        add(b->p, F);
    add(e->ring.p, (size_t)nsamp * e->ps.row_doubles * sizeof(double));
    add(e->d_fd.p, e->d_fd.n * sizeof(double));
    add(e->d_fd_count.p, sizeof(int));
    add(e->mur_buf.p, e->mur_buf.n * sizeof(float));
    add(e->rlc_state.p, e->rlc_state.n * sizeof(float));
    for (DevBuf<float>* b : {&e->AVx, &e->LVx, &e->AIx, &e->LIx}) add(b->p, b->n * sizeof(float));
    return v;
}

void ckpt_header(const fdtd_engine_s* e, uint32_t nsamp, CkptHeader& h) {
    std::memset(&h, 0, sizeof(h));
    std::memcpy(h.magic, "WFDTDCK1", 8);
    h.version = 2;
    for (int a = 0; a < 3; ++a) h.N[a] = e->N[a];
    h.Nzp = e->Nzp;
    // the sample row layout from the host's probe columns (known before the
    // probes are uploaded, so a blob can be checked before anything changes)
    h.nprobe = (uint32_t)e->h_weight.size();
    h.row_doubles = 2 + h.nprobe;
    h.nfreq = (uint32_t)e->h_freq.size();
    h.nmur = (uint32_t)e->mur.nface;
    h.ts = e->ts;
    h.done = e->done ? 1u : 0u;
    h.nsamp = nsamp;
    h.frame = (e->fused ? 1 : 0) | (e->rot << 1);
    h.nrlc = e->rlc.count;
}
}  // namespace

int fdtd_engine_checkpoint(fdtd_engine_t e, void* buf, uint64_t cap, uint64_t* size) {
    if (!e || !size) return FDTD_ERR_ARG;
    if (e->pending) {
        set_error("fdtd_engine_checkpoint: wait for the asynchronous iterate first");
        return FDTD_ERR_STATE;
    }
    CK(cudaSetDevice(e->device));
    int rc;
    if ((rc = start(e))) return rc;  // a checkpoint of a fresh engine holds its ts = 0 sample
    int ctl[4] = {0, 0, 0, 0};
    CK(cudaMemcpyAsync(ctl, e->ctl.p, sizeof(ctl), cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    const uint32_t nsamp = (uint32_t)ctl[1];
    const std::vector<CkptPart> parts = ckpt_parts(e, nsamp);
    uint64_t need = sizeof(CkptHeader);
    for (const CkptPart& q : parts) need += sizeof(uint64_t) + q.bytes;
    *size = need;
    if (!buf) return FDTD_OK;  // size query
    if (cap < need) {
        set_error("fdtd_engine_checkpoint: buffer too small");
        return FDTD_ERR_ARG;
    }
    CkptHeader h;
    ckpt_header(e, nsamp, h);
    char* o = static_cast<char*>(buf);
    std::memcpy(o, &h, sizeof(h));
    o += sizeof(h);
    for (const CkptPart& q : parts) {
        const uint64_t b = q.bytes;
        std::memcpy(o, &b, sizeof(b));
        o += sizeof(b);
        if (b) CK(cudaMemcpyAsync(o, q.p, b, cudaMemcpyDeviceToHost, e->stream));
        o += b;
    }
    CK(cudaStreamSynchronize(e->stream));
    return FDTD_OK;
}

// Restore validates the whole blob -- header, sample count and every part's
// size against this engine, and the blob's length -- before it changes
// anything: a rejected blob leaves the engine exactly as it was (a fresh
// engine keeps its pending ts = 0 sample and FD accumulation).  Only then
// are the parts copied to the device.
int fdtd_engine_restore(fdtd_engine_t e, const void* buf, uint64_t size) {
    if (!e || !buf) return FDTD_ERR_ARG;
    if (e->pending) {
        set_error("fdtd_engine_restore: wait for the asynchronous iterate first");
        return FDTD_ERR_STATE;
    }
    if (size < sizeof(CkptHeader)) {
        set_error("fdtd_engine_restore: blob too small");
        return FDTD_ERR_ARG;
    }
    CkptHeader h;
    std::memcpy(&h, buf, sizeof(h));
    CkptHeader mine;
    ckpt_header(e, h.nsamp, mine);
    if (std::memcmp(h.magic, mine.magic, 8) != 0 || h.version != mine.version || h.N[0] != mine.N[0] ||
        h.N[1] != mine.N[1] || h.N[2] != mine.N[2] || h.Nzp != mine.Nzp || h.nprobe != mine.nprobe ||
        h.row_doubles != mine.row_doubles || h.nfreq != mine.nfreq || h.nmur != mine.nmur || h.frame != mine.frame ||
        h.nrlc != mine.nrlc) {
        set_error("fdtd_engine_restore: the checkpoint belongs to a different engine configuration");
        return FDTD_ERR_ARG;
    }
    if (h.nsamp > (uint32_t)e->cap) {
        set_error("fdtd_engine_restore: the checkpoint holds more samples than this engine's ring");
        return FDTD_ERR_ARG;
    }
    CK(cudaSetDevice(e->device));
    int rc;
    // the probe tables and the sample ring (idempotent; no simulation state)
    if ((rc = upload_probes(e))) return rc;
    const std::vector<CkptPart> parts = ckpt_parts(e, h.nsamp);
    const char* const first = static_cast<const char*>(buf) + sizeof(h);
    const char* const end = static_cast<const char*>(buf) + size;
    // pass 1: every (bytes, payload) pair and the total length
    const char* o = first;
    for (const CkptPart& q : parts) {
        uint64_t b = 0;
        if ((size_t)(end - o) < sizeof(b)) {
            set_error("fdtd_engine_restore: blob truncated");
            return FDTD_ERR_ARG;
        }
        std::memcpy(&b, o, sizeof(b));
        o += sizeof(b);
        if (b != q.bytes || (uint64_t)(end - o) < b) {
            set_error("fdtd_engine_restore: a state array does not match this engine");
            return FDTD_ERR_ARG;
        }
        o += b;
    }
    if (o != end) {
        set_error("fdtd_engine_restore: trailing bytes after the last state array");
        return FDTD_ERR_ARG;
    }
    // pass 2: the blob is sound; replace the state
    if (!e->started) e->need_initial_sample = false;  // the blob holds the samples
    if ((rc = start(e))) return rc;
    o = first;
    for (const CkptPart& q : parts) {
        uint64_t b = 0;
        std::memcpy(&b, o, sizeof(b));
        o += sizeof(b);
        if (b) CK(cudaMemcpyAsync(q.p, o, b, cudaMemcpyHostToDevice, e->stream));
        o += b;
    }
    CK(cudaStreamSynchronize(e->stream));
    e->ts = h.ts;
    e->done = h.done != 0;
    e->need_initial_sample = false;
    return FDTD_OK;
}

int fdtd_engine_query(fdtd_engine_t e, int* ready) {
    if (!e || !ready) return FDTD_ERR_ARG;
    if (!e->pending) {
        *ready = 1;
        return FDTD_OK;
    }
    CK(cudaSetDevice(e->device));
    const cudaError_t q = cudaEventQuery(e->ev1);
    if (q == cudaErrorNotReady) {
        *ready = 0;
        return FDTD_OK;
    }
    if (q != cudaSuccess) {
        set_error(std::string("fdtd_engine_query: ") + cudaGetErrorString(q));
        return FDTD_ERR_CUDA;
    }
    *ready = 1;
    return FDTD_OK;
}

int fdtd_engine_done(fdtd_engine_t e, int* done) {
    if (!e || !done) return FDTD_ERR_ARG;
    *done = e->done ? 1 : 0;
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
    CK(cudaMemcpyAsync(&v, e->p_nsamp(), sizeof(int), cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    *n = (uint32_t)v;
    return FDTD_OK;
}

int fdtd_engine_read_samples(fdtd_engine_t e, uint32_t first, uint32_t count, uint32_t* ts, double* vals,
                             double* energy) {
    if (!e) return FDTD_ERR_ARG;
    uint32_t n = 0;
    const int rc = fdtd_engine_num_samples(e, &n);
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
    if (e->pending) {
        set_error("fdtd_engine_energy: wait for the asynchronous iterate first");
        return FDTD_ERR_STATE;
    }
    CK(cudaSetDevice(e->device));
    DevGrid g = e->g;
    g.V = e->cur_V();
    g.I = e->cur_I();
    // the segments, plane sums and total of a sample step, from the fields
    const dim3 grid((unsigned)g.nzt, (e->N[1] - 1 + 7) / 8, e->N[0] - 1);
    k_energy_segments<<<grid, dim3(32, 8), 0, e->stream>>>(g);
    k_energy_planes<<<e->N[0] - 1, 256, 0, e->stream>>>(g);
    k_energy_total<<<1, 32, 0, e->stream>>>(g, kEps0, kMue0, e->d_energy_tmp.p);
    CK(cudaGetLastError());
    double h = 0;
    CK(cudaMemcpyAsync(&h, e->d_energy_tmp.p, sizeof(h), cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    *energy = h;
    return FDTD_OK;
}

int fdtd_engine_get_fields(fdtd_engine_t e, float* volt, float* curr) {
    if (!e) return FDTD_ERR_ARG;
    CK(cudaSetDevice(e->device));
    const uint32_t Nx = e->N[0], Ny = e->N[1], Nz = e->N[2];
    const size_t n = (size_t)3 * Nx * Ny * Nz;
    std::vector<float> tmp(e->rot ? n : 0);
    for (int which = 0; which < 2; ++which) {
        float* dst = which ? curr : volt;
        if (!dst) continue;
        const float* src = which ? e->cur_I() : e->cur_V();
        // rows of Nz floats out of rows of Nzp floats
        CK(cudaMemcpy2DAsync(e->rot ? tmp.data() : dst, Nz * sizeof(float), src, e->Nzp * sizeof(float),
                             Nz * sizeof(float), (size_t)3 * Nx * Ny, cudaMemcpyDeviceToHost, e->stream));
        if (!e->rot) continue;
        CK(cudaStreamSynchronize(e->stream));
        // device [3][Nx][Ny][Nz] -> the operator's [3][N0x][N0y][N0z]
        const uint32_t* M = e->N0;
        const size_t NN = (size_t)M[0] * M[1] * M[2];
        for (int c = 0; c < 3; ++c) {
            const float* s = tmp.data() + (size_t)e->dev_comp(c) * Nx * Ny * Nz;
            float* d = dst + c * NN;
            uint32_t o[3], dv[3];
            for (o[0] = 0; o[0] < M[0]; ++o[0])
                for (o[1] = 0; o[1] < M[1]; ++o[1])
                    for (o[2] = 0; o[2] < M[2]; ++o[2]) {
                        e->dev_node(o, dv);
                        *d++ = s[((size_t)dv[0] * Ny + dv[1]) * Nz + dv[2]];
                    }
        }
    }
    CK(cudaStreamSynchronize(e->stream));
    return FDTD_OK;
}

int fdtd_engine_dump_field(fdtd_engine_t e, const fdtd_dump_box* b, float* out, uint64_t cap, uint32_t num[3]) {
    if (!e || !b || !num) return FDTD_ERR_ARG;
    if (b->field < 0 || b->field > 1 || b->interp < 0 || b->interp > 2) {
        set_error("fdtd_engine_dump_field: field must be 0 (E) or 1 (H), interp 0 (none), 1 (node) or 2 (cell)");
        return FDTD_ERR_ARG;
    }
    DumpBox d{};  // in device axes (the interpolation is written per component n, nP, nPP)
    d.field = b->field;
    d.interp = b->interp;
    uint64_t total = 1;
    for (int a = 0; a < 3; ++a) {  // the operator's axis a is device axis dev_comp(a)
        const uint32_t lo = std::min(b->start[a], b->stop[a]), hi = std::max(b->start[a], b->stop[a]);
        if (hi >= e->N0[a]) {
            set_error("fdtd_engine_dump_field: box outside the grid");
            return FDTD_ERR_ARG;
        }
        const uint32_t step = b->step[a] ? b->step[a] : 1;
        num[a] = (hi - lo) / step + 1;  // ProcessFields::CalcMeshPos, SUBSAMPLE
        const int da = e->dev_comp(a);
        d.start[da] = (int)lo;
        d.step[da] = (int)step;
        d.num[da] = (int)num[a];
        total *= num[a];
    }
    if (!out) return FDTD_OK;  // size query
    if (cap < 3 * total) {
        set_error("fdtd_engine_dump_field: output buffer too small");
        return FDTD_ERR_ARG;
    }
    if (!e->edges.p) {
        set_error("fdtd_engine_dump_field: the operator description had no mesh lines (edge lengths unknown)");
        return FDTD_ERR_STATE;
    }
    if (e->pending) {
        set_error("fdtd_engine_dump_field: wait for the asynchronous iterate first");
        return FDTD_ERR_STATE;
    }
    CK(cudaSetDevice(e->device));
    int rc;
    if ((rc = start(e))) return rc;
    if (e->dump.n < 3 * total) {
        if (e->dump.p) {
            e->device_bytes -= e->dump.n * sizeof(float);
            e->dump.release();
        }
        if ((rc = e->dump.alloc(3 * total, e->device_bytes, e->stream))) return rc;
    }
    const unsigned blocks = (unsigned)std::min<uint64_t>((total + 255) / 256, 4096);
    k_dump_field<<<blocks, 256, 0, e->stream>>>(e->g, e->cur_V(), e->cur_I(), e->edges.p, d, e->dump.p);
    if ((rc = check_launch())) return rc;
    if (!e->rot) {
        CK(cudaMemcpyAsync(out, e->dump.p, 3 * total * sizeof(float), cudaMemcpyDeviceToHost, e->stream));
        CK(cudaStreamSynchronize(e->stream));
        return FDTD_OK;
    }
    std::vector<float> tmp(3 * total);
    CK(cudaMemcpyAsync(tmp.data(), e->dump.p, 3 * total * sizeof(float), cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    // device [3][d.num] -> the operator's [3][num]
    for (int c = 0; c < 3; ++c) {
        const float* s = tmp.data() + (size_t)e->dev_comp(c) * total;
        float* o = out + (size_t)c * total;
        uint32_t i[3], j[3];
        for (i[0] = 0; i[0] < num[0]; ++i[0])
            for (i[1] = 0; i[1] < num[1]; ++i[1])
                for (i[2] = 0; i[2] < num[2]; ++i[2]) {
                    e->dev_node(i, j);
                    *o++ = s[((size_t)j[0] * d.num[1] + j[1]) * d.num[2] + j[2]];
                }
    }
    return FDTD_OK;
}

static int get_one(fdtd_engine_t e, const float* base, uint32_t n, uint32_t x, uint32_t y, uint32_t z, float* v) {
    if (!e || !v || n > 2 || x >= e->N0[0] || y >= e->N0[1] || z >= e->N0[2]) {
        set_error("field access out of range");
        return FDTD_ERR_ARG;
    }
    CK(cudaSetDevice(e->device));
    const uint32_t o[3] = {x, y, z};
    const long long off = e->dev_comp((int)n) * e->comp + e->dev_offset(o);
    CK(cudaMemcpyAsync(v, base + off, sizeof(float), cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    return FDTD_OK;
}

int fdtd_engine_get_volt(fdtd_engine_t e, uint32_t n, uint32_t x, uint32_t y, uint32_t z, float* v) {
    return get_one(e, e ? e->cur_V() : nullptr, n, x, y, z, v);
}
int fdtd_engine_get_curr(fdtd_engine_t e, uint32_t n, uint32_t x, uint32_t y, uint32_t z, float* v) {
    return get_one(e, e ? e->cur_I() : nullptr, n, x, y, z, v);
}

static int set_one(fdtd_engine_t e, float* base, uint32_t n, uint32_t x, uint32_t y, uint32_t z, float v) {
    if (!e || n > 2 || x >= e->N0[0] || y >= e->N0[1] || z >= e->N0[2]) {
        set_error("field access out of range");
        return FDTD_ERR_ARG;
    }
    if (e->pending) {
        set_error("field write: wait for the asynchronous iterate first");
        return FDTD_ERR_STATE;
    }
    CK(cudaSetDevice(e->device));
    const uint32_t o[3] = {x, y, z};
    const long long off = e->dev_comp((int)n) * e->comp + e->dev_offset(o);
    CK(cudaMemcpyAsync(base + off, &v, sizeof(float), cudaMemcpyHostToDevice, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    return FDTD_OK;
}
int fdtd_engine_set_volt(fdtd_engine_t e, uint32_t n, uint32_t x, uint32_t y, uint32_t z, float v) {
    return set_one(e, e ? e->cur_V() : nullptr, n, x, y, z, v);
}
int fdtd_engine_set_curr(fdtd_engine_t e, uint32_t n, uint32_t x, uint32_t y, uint32_t z, float v) {
    return set_one(e, e ? e->cur_I() : nullptr, n, x, y, z, v);
}

int fdtd_engine_probe_now(fdtd_engine_t e, const fdtd_probe_desc* p, double* value) {
    if (!e || !p || !value || (p->type != 0 && p->type != 1)) {
        set_error("fdtd_engine_probe_now: a voltage (0) or current (1) probe is needed");
        return FDTD_ERR_ARG;
    }
    if (e->pending) {
        set_error("fdtd_engine_probe_now: wait for the asynchronous iterate first");
        return FDTD_ERR_STATE;
    }
    std::vector<ProbeEntry> ent;
    int rc = probe_entries(e, p, ent);
    if (rc) return rc;
    *value = 0.0;
    if (ent.empty()) return FDTD_OK;
    CK(cudaSetDevice(e->device));
    uint64_t& tb = e->device_bytes;
    if (e->now_entries.n < ent.size()) {
        e->now_entries.release();
        if ((rc = e->now_entries.alloc(ent.size(), tb, e->stream))) return rc;
    }
    if (!e->now_misc.p && (rc = e->now_misc.alloc(4, tb, e->stream))) return rc;
    // now_misc: [0] the sum, [1] div = 0 (an integral), [2..3] first = {0, count} as ints
    double misc[4] = {0.0, 0.0, 0.0, 0.0};
    int first[2] = {0, (int)ent.size()};
    std::memcpy(&misc[2], first, sizeof(first));
    CK(cudaMemcpyAsync(e->now_entries.p, ent.data(), ent.size() * sizeof(ProbeEntry), cudaMemcpyHostToDevice,
                       e->stream));
    CK(cudaMemcpyAsync(e->now_misc.p, misc, sizeof(misc), cudaMemcpyHostToDevice, e->stream));
    ProbeSet ps{};
    ps.entries = e->now_entries.p;
    ps.first = reinterpret_cast<const int*>(e->now_misc.p + 2);
    ps.div = e->now_misc.p + 1;
    ps.nprobe = 1;
    DevGrid g = e->g;
    g.V = e->cur_V();
    g.I = e->cur_I();
    g.V2 = nullptr;  // the current buffers are named directly
    k_probe_now<<<1, 32, 0, e->stream>>>(ps, g, e->now_misc.p);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(value, e->now_misc.p, sizeof(double), cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    return FDTD_OK;
}

int fdtd_engine_profile_kernels(fdtd_engine_t e, uint32_t n_steps, double* ms_volt, double* ms_curr) {
    if (!e || n_steps == 0) return FDTD_ERR_ARG;
    CK(cudaSetDevice(e->device));
    int rc;
    if ((rc = start(e))) return rc;
    std::vector<cudaEvent_t> ev(3 * (size_t)n_steps);
    for (auto& x : ev) CK(cudaEventCreate(&x));
    for (uint32_t k = 0; k < n_steps; ++k) {
        const bool sample = e->interval && ((e->ts + 1) % e->interval) == 0;
        CK(cudaEventRecord(ev[3 * k], e->stream));
        if (e->fused) {  // one kernel per step: reported as the "volt" time
            launch_fused(e, 0, sample && e->energy_on_probe);
            CK(cudaEventRecord(ev[3 * k + 1], e->stream));
        } else {
            launch_volt_hooks(e, 0);
            CK(cudaEventRecord(ev[3 * k + 1], e->stream));
            launch_curr(e, 0, sample && e->energy_on_probe);
        }
        CK(cudaEventRecord(ev[3 * k + 2], e->stream));
        if ((rc = check_launch())) return rc;
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
    return check_error_word(e);
}

int fdtd_engine_get_stats(fdtd_engine_t e, fdtd_engine_stats* st) {
    if (!e || !st) return FDTD_ERR_ARG;
    std::memset(st, 0, sizeof(*st));
    st->num_tuples = std::max(e->num_tuples_e, e->num_tuples_h);
    st->index_bytes = (e->E.idx16 && e->H.idx16) ? 2 : 4;
    st->num_upml_nodes = e->upml_nodes;
    st->num_ade_nodes = e->ade_nodes;
    st->padded_nz = (uint32_t)e->Nzp;
    st->device_bytes = e->device_bytes;
    st->tile_y = (uint32_t)(e->fused ? FU_TY : (e->use_tma ? e->tma_ty : e->TY));
    st->x_chunk = (uint32_t)e->XC;
    st->kernel = e->fused ? 2u : (e->use_tma ? 3u : 1u);
    return FDTD_OK;
}

int fdtd_engine_last_timing(fdtd_engine_t e, double* ms, uint64_t* launches) {
    if (!e) return FDTD_ERR_ARG;
    if (ms) *ms = e->last_ms;
    if (launches) *launches = e->last_launches;
    return FDTD_OK;
}

}  // extern "C"
