// Kernel launch templates of the single-engine kernel families (TMA ring
// and direct), shared by engine.cu (feature sets 0..3) and engine_adex.cu
// (the variants with Lorentz/Drude dispersion orders 1..3, compiled in their
// own translation unit so the two build in parallel).
#pragma once

#include <cuda_runtime.h>

#include "engine_state.h"

namespace wipems {

template <typename IdxT, int FEAT, bool GEO, int TY>
void launch_volt_tma(fdtd_engine_s* e, int ts_off) {
    constexpr bool UP = (FEAT & FEAT_UPML) != 0;
    const size_t sm = StageLayout<IdxT, UP, (FEAT & FEAT_ADE) != 0, TY>::smem(e->stages);
    dim3 grid((e->ti.ne[2] + 31) / 32, (e->ti.ne[1] + TY - 1) / TY, (e->ti.ne[0] + e->XC - 1) / e->XC);
    k_volt_tma<IdxT, FEAT, GEO, TY><<<grid, dim3(32, TY), sm, e->stream>>>(e->g, e->maps, e->ti, ts_off, e->XC,
                                                                           e->stages);
}

template <typename IdxT, int FEAT, bool GEO, bool EN, int TY>
void launch_curr_tma(fdtd_engine_s* e, int ts_off) {
    constexpr bool UP = (FEAT & FEAT_UPML) != 0;
    const size_t sm = StageLayout<IdxT, UP, false, TY>::smem(e->stages);
    dim3 grid((e->N[2] - 1 + 31) / 32, (e->N[1] - 1 + TY - 1) / TY, (e->N[0] - 1 + e->XC - 1) / e->XC);
    k_curr_tma<IdxT, FEAT, GEO, EN, TY><<<grid, dim3(32, TY), sm, e->stream>>>(e->g, e->maps, e->ti, ts_off, e->XC,
                                                                               e->stages);
}

template <typename IdxT, int FEAT, bool GEO>
void launch_volt_t(fdtd_engine_s* e, int ts_off) {
    if (e->use_tma) {
        if (e->tma_ty == 8) launch_volt_tma<IdxT, FEAT, GEO, 8>(e, ts_off);
        else launch_volt_tma<IdxT, FEAT, GEO, TMA_TY>(e, ts_off);
    } else {
        dim3 grid((e->N[2] + 31) / 32, (e->N[1] + e->TY - 1) / e->TY, (e->N[0] + e->XC - 1) / e->XC);
        k_volt<IdxT, FEAT, GEO><<<grid, dim3(32, e->TY), e->smem_direct, e->stream>>>(e->g, ts_off, e->XC);
    }
}

template <typename IdxT, int FEAT, bool GEO, bool EN>
void launch_curr_t(fdtd_engine_s* e, int ts_off) {
    if (e->use_tma) {
        if (e->tma_ty == 8) launch_curr_tma<IdxT, FEAT, GEO, EN, 8>(e, ts_off);
        else launch_curr_tma<IdxT, FEAT, GEO, EN, TMA_TY>(e, ts_off);
    } else {
        dim3 grid((e->N[2] + 31) / 32, (e->N[1] + e->TY - 1) / e->TY, (e->N[0] - 1 + e->XC - 1) / e->XC);
        k_curr<IdxT, FEAT, GEO, EN><<<grid, dim3(32, e->TY), e->smem_direct, e->stream>>>(e->g, ts_off, e->XC);
    }
}

template <typename IdxT, int FEAT, bool GEO>
cudaError_t smem_attr_one(int bytes) {
    const cudaFuncAttribute a = cudaFuncAttributeMaxDynamicSharedMemorySize;
    cudaError_t r[6] = {cudaFuncSetAttribute(k_volt_tma<IdxT, FEAT, GEO, TMA_TY>, a, bytes),
                        cudaFuncSetAttribute(k_curr_tma<IdxT, FEAT, GEO, true, TMA_TY>, a, bytes),
                        cudaFuncSetAttribute(k_curr_tma<IdxT, FEAT, GEO, false, TMA_TY>, a, bytes),
                        cudaFuncSetAttribute(k_volt_tma<IdxT, FEAT, GEO, 8>, a, bytes),
                        cudaFuncSetAttribute(k_curr_tma<IdxT, FEAT, GEO, true, 8>, a, bytes),
                        cudaFuncSetAttribute(k_curr_tma<IdxT, FEAT, GEO, false, 8>, a, bytes)};
    for (cudaError_t x : r)
        if (x != cudaSuccess) return x;
    return cudaSuccess;
}


// engine_adex.cu: feature sets FEAT_ADE | FEAT_ADEX (+ FEAT_UPML), chosen by e->feat
template <typename IdxT, bool GEO>
void launch_volt_adex(fdtd_engine_s* e, int ts_off);
template <typename IdxT, bool GEO, bool EN>
void launch_curr_adex(fdtd_engine_s* e, int ts_off);
cudaError_t smem_attrs_adex(int bytes);

}  // namespace wipems
