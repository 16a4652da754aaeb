// The kernel variants for Lorentz/Drude dispersion of order > 1 (feature
// sets FEAT_ADE | FEAT_ADEX with and without UPML), instantiated here so
// that they compile in parallel with engine.cu.
#include "launch.cuh"

namespace wipems {

template <typename IdxT, bool GEO>
void launch_volt_adex(fdtd_engine_s* e, int ts_off) {
    if (e->feat & FEAT_UPML) launch_volt_t<IdxT, FEAT_UPML | FEAT_ADE | FEAT_ADEX, GEO>(e, ts_off);
    else launch_volt_t<IdxT, FEAT_ADE | FEAT_ADEX, GEO>(e, ts_off);
}

template <typename IdxT, bool GEO, bool EN>
void launch_curr_adex(fdtd_engine_s* e, int ts_off) {
    if (e->feat & FEAT_UPML) launch_curr_t<IdxT, FEAT_UPML | FEAT_ADE | FEAT_ADEX, GEO, EN>(e, ts_off);
    else launch_curr_t<IdxT, FEAT_ADE | FEAT_ADEX, GEO, EN>(e, ts_off);
}

cudaError_t smem_attrs_adex(int bytes) {
    cudaError_t r = cudaSuccess, t;
#define WIPEMS_ATTR(I, F)                                                 \
    if ((t = smem_attr_one<I, F, false>(bytes)) != cudaSuccess) r = t;    \
    if ((t = smem_attr_one<I, F, true>(bytes)) != cudaSuccess) r = t;
    WIPEMS_ATTR(uint16_t, 6) WIPEMS_ATTR(uint16_t, 7) WIPEMS_ATTR(uint32_t, 6) WIPEMS_ATTR(uint32_t, 7)
#undef WIPEMS_ATTR
    return r;
}

template void launch_volt_adex<uint16_t, false>(fdtd_engine_s*, int);
template void launch_volt_adex<uint16_t, true>(fdtd_engine_s*, int);
template void launch_volt_adex<uint32_t, false>(fdtd_engine_s*, int);
template void launch_volt_adex<uint32_t, true>(fdtd_engine_s*, int);
template void launch_curr_adex<uint16_t, false, false>(fdtd_engine_s*, int);
template void launch_curr_adex<uint16_t, false, true>(fdtd_engine_s*, int);
template void launch_curr_adex<uint16_t, true, false>(fdtd_engine_s*, int);
template void launch_curr_adex<uint16_t, true, true>(fdtd_engine_s*, int);
template void launch_curr_adex<uint32_t, false, false>(fdtd_engine_s*, int);
template void launch_curr_adex<uint32_t, false, true>(fdtd_engine_s*, int);
template void launch_curr_adex<uint32_t, true, false>(fdtd_engine_s*, int);
template void launch_curr_adex<uint32_t, true, true>(fdtd_engine_s*, int);

}  // namespace wipems
