// Per-node fused update of one half-step, shared by the direct and the
// TMA-pipelined kernels.
//
// Per-cell math restated from the reference (citations relative to it):
//   voltage update   FDTD/engine.cpp:108-161 (SSE twin engine_sse_compressed.cpp:48-156)
//   current update   FDTD/engine.cpp:163-210 (SSE twin engine_sse_compressed.cpp:158-263)
//   UPML flux swap   extensions/engine_ext_upml.cpp:57-239, fused as
//                      f  = vvp*V - vvfo*F                     (pre)
//                      Fn = F*vv + vi*curl                     (main, V<-F)
//                      V  = f + vvfn*Fn ; F = Fn               (post)
//   Lorentz/Drude    extensions/engine_ext_lorentzmaterial.cpp:79-173 (pre, old V)
//                    extensions/engine_ext_dispersive.cpp:76-132 (V -= ADE after)
//   excitation       extensions/engine_ext_excitation.cpp:33-99 (added last)
// Hook order per half-step follows Engine::IterateTS (engine.cpp:255-274)
// with the priorities of engine_extension.h:21-29: ADE-pre, UPML-pre, main,
// UPML-post, ADE-apply, excitation.  Every product and sum is rounded in the
// reference's order (__fmul_rn/__fadd_rn, no FMA contraction), so the device
// result is bit-identical to the FP32 CPU engine (up to the geometry factor
// product on graded meshes, see cop.h).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "cop.h"

namespace wipems {

// kernel feature bits (compile time)
constexpr int FEAT_UPML = 1;
constexpr int FEAT_ADE = 2;
constexpr int FEAT_ADEX = 4;  // dispersion orders 1..3 (always with FEAT_ADE)

// device view of one half-step's tables (float4 units, layout TAB_* in cop.h)
struct DevHalf {
    const void* idx;     // [Nx][Ny][Nzp] tuple index (uint16 or uint32)
    const float4* main;
    const float4* upml;
    const float4* ade;
    const float4* exc;
    const float4* adex;  // dispersion orders 1..3: [order-1][tuple][TAB_ADE] or null
    int ntup;            // tuples in the table (the adex order stride)
};

struct DevGrid {
    int Nx, Ny, Nz;      // mesh lines
    int Nzp;             // padded z stride (multiple of 32)
    long long sx;        // x stride (Ny*Nzp)
    long long comp;      // component stride (Nx*Ny*Nzp)
    float* V;            // [3][comp]
    float* I;            // [3][comp]
    float* FV;           // UPML voltage flux [3][comp] or null
    float* FI;           // UPML current flux
    float* V2;           // fused single-pass kernel: second field buffers
    float* I2;           // (fields at numTS live in V/I when numTS is even,
    float* FV2;          // in V2/I2 when odd); null otherwise
    float* AV;           // ADE voltage state (order 1) [3][comp]
    float* LV;           // Lorentz voltage state
    float* AI;           // ADE current state
    float* LI;
    // states of dispersion orders 1..3: [order-1][3][comp] (null when the
    // operator has order 1 only)
    float* AVx;
    float* LVx;
    float* AIx;
    float* LIx;
    // per (x, 8-row y tile, 32-node z tile) of the voltage kernel: bit 0 =
    // a Lorentz/Drude node, bit 1 = a Lorentz node in that tile plane
    // (the TMA kernels stage the states of those tile planes); null = none
    const uint8_t* ade_tile;
    DevHalf e, h;
    const float* geo;    // [4][Nx+Ny+Nz] dE, iD, dH, iM (factorized meshes) or null
    int geo_stride;      // Nx+Ny+Nz
    const float* sigV;   // excitation signals
    const float* sigC;
    int sig_len;
    int sig_period;      // 0 = none
    const int* d_ts;     // timestep counter (numTS)
    const int* d_done;   // set once the job met its end criterion: kernels skip
    double* d_eacc;      // [2]: running energy maximum (end criterion)
    // energy on sample steps, in an order fixed by the grid alone: one
    // (sum V^2, sum I^2) float pair per segment (x < Nx-1, y < Ny-1, 32-node
    // z tile zt < nzt) written by the warp that updates it, then one double
    // pair per x plane (k_energy_planes), summed in x order by the sampler
    float2* eseg;        // [(Nx-1)*(Ny-1)*nzt]
    double2* eplane;     // [Nx-1]
    int nzt;             // ceil((Nz-1)/32)
};

// One energy segment: the 32 z-lanes of a warp at plane x, row y, z tile zt.
// Each lane squares its V and I components (float products, summed in
// component order), a fixed shuffle tree adds the 32 lanes, and lane 0
// stores the pair.  Every lane of the warp calls this (act = the lane's node
// counts: z < Nz-1 and the update ran); `owner` = the segment exists
// (y < Ny-1, zt < nzt) and this warp is the one that writes it.
__device__ __forceinline__ void energy_segment(const DevGrid& g, int x, int y, int zt, bool act, bool owner,
                                               float v0, float v1, float v2, float i0, float i1, float i2) {
    float pe = 0.f, ph = 0.f;
    if (act) {
        pe = __fadd_rn(__fadd_rn(__fmul_rn(v0, v0), __fmul_rn(v1, v1)), __fmul_rn(v2, v2));
        ph = __fadd_rn(__fadd_rn(__fmul_rn(i0, i0), __fmul_rn(i1, i1)), __fmul_rn(i2, i2));
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        pe = __fadd_rn(pe, __shfl_down_sync(0xffffffffu, pe, off));
        ph = __fadd_rn(ph, __shfl_down_sync(0xffffffffu, ph, off));
    }
    if (owner && (threadIdx.x & 31) == 0)
        g.eseg[((long long)x * (g.Ny - 1) + y) * g.nzt + zt] = make_float2(pe, ph);
}

template <typename IdxT>
__device__ __forceinline__ uint32_t load_idx(const void* p, long long o) {
    return (uint32_t)__ldg(reinterpret_cast<const IdxT*>(p) + o);
}

__device__ __forceinline__ int exc_index(int numTS, int delay, int length, int period) {
    // engine_ext_excitation.cpp:44-53
    int exc_pos = numTS - delay;
    exc_pos *= (exc_pos > 0);
    const int p = period > 0 ? period : numTS + 1;
    exc_pos %= p;
    exc_pos *= (exc_pos < length);
    return exc_pos;
}

// geometry factors of one node for the three components (factorized meshes):
// E: gE(n) = dE[n][p_n] * iD[nP][p_nP] * iD[nPP][p_nPP]; H with dH / iM.
struct GeoF {
    float f[3][3];
};

__device__ __forceinline__ GeoF geo_factors(const DevGrid& g, bool H, int x, int y, int z) {
    const int S = g.geo_stride;
    const float* a = g.geo + (H ? 2 : 0) * S;  // dE | dH
    const float* b = g.geo + (H ? 3 : 1) * S;  // iD | iM
    const int p[3] = {x, g.Nx + y, g.Nx + g.Ny + z};
    GeoF r;
#pragma unroll
    for (int n = 0; n < 3; ++n) {
        r.f[n][0] = __ldg(a + p[n]);
        r.f[n][1] = __ldg(b + p[(n + 1) % 3]);
        r.f[n][2] = __ldg(b + p[(n + 2) % 3]);
    }
    return r;
}

// One node of one half-step.  fld[3]: the old field (V or I); curl[3]: the
// curl of the other field; t: tuple index; o: node offset; F (UPML flux of
// the node) is read from fsrc[n*fstride] when fsrc is set, else from global.
// The new flux goes to fout (default: the engine's flux array, in place),
// and only when fwrite is set.  The Lorentz/Drude states are read from
// asrc / lsrc[n*fstride] when set (staged copies), else from global; the
// new states always go to global.
template <bool H, int FEAT, bool GEO>
__device__ __forceinline__ void update_node(const DevGrid& g, float fld[3], const float curl[3], uint32_t t,
                                            long long o, int numTS, const float* fsrc, int fstride,
                                            const GeoF& gf, float* fout = nullptr, bool fwrite = true,
                                            const float* asrc = nullptr, const float* lsrc = nullptr) {
    const DevHalf& T = H ? g.h : g.e;
    const float4 ta = __ldg(&T.main[TAB_MAIN * t]);
    const float4 tb = __ldg(&T.main[TAB_MAIN * t + 1]);
    const float c1[3] = {ta.x, ta.y, ta.z};
    float c2[3] = {ta.w, tb.x, tb.y};
    if (GEO) {
#pragma unroll
        for (int n = 0; n < 3; ++n) c2[n] = __fmul_rn(__fmul_rn(__fmul_rn(c2[n], gf.f[n][0]), gf.f[n][1]), gf.f[n][2]);
    }
    // In tile planes that hold Lorentz/Drude nodes (the staged state
    // pointer is set) the ADE coefficients are loaded with the main tuple,
    // not after its flags: one table round trip per node instead of two.
    const bool spec_a = (FEAT & FEAT_ADE) && asrc != nullptr;
    float4 sa0 = make_float4(0.f, 0.f, 0.f, 0.f), sa1 = sa0, sa2 = sa0;
    if (spec_a) {
        sa0 = __ldg(&T.ade[TAB_ADE * t]);
        sa1 = __ldg(&T.ade[TAB_ADE * t + 1]);
        sa2 = __ldg(&T.ade[TAB_ADE * t + 2]);
    }
    const uint32_t flags = __float_as_uint(tb.z);
    const long long C = g.comp;
    float* A = H ? g.AI : g.AV;
    float* Lr = H ? g.LI : g.LV;
    float* Fl = fout ? fout : (H ? g.FI : g.FV);
    float ade[3] = {0.f, 0.f, 0.f};
    if ((FEAT & FEAT_ADE) && (flags & TF_ADE)) {
        const float4 a0 = spec_a ? sa0 : __ldg(&T.ade[TAB_ADE * t]);
        const float4 a1 = spec_a ? sa1 : __ldg(&T.ade[TAB_ADE * t + 1]);
        const float4 a2 = spec_a ? sa2 : __ldg(&T.ade[TAB_ADE * t + 2]);
        const float kint[3] = {a0.x, a0.y, a0.z};
        const float kext[3] = {a0.w, a1.x, a1.y};
        const float klor[3] = {a1.z, a1.w, a2.x};
        if (flags & TF_LOR) {
#pragma unroll
            for (int n = 0; n < 3; ++n) {
                float lor = lsrc ? lsrc[n * fstride] : Lr[n * C + o];
                float a = asrc ? asrc[n * fstride] : A[n * C + o];
                lor = __fadd_rn(lor, __fmul_rn(klor[n], a));
                a = __fmul_rn(a, kint[n]);
                a = __fadd_rn(a, __fmul_rn(kext[n], __fsub_rn(fld[n], lor)));
                Lr[n * C + o] = lor;
                A[n * C + o] = a;
                ade[n] = a;
            }
        } else {
#pragma unroll
            for (int n = 0; n < 3; ++n) {
                float a = asrc ? asrc[n * fstride] : A[n * C + o];
                a = __fmul_rn(a, kint[n]);
                a = __fadd_rn(a, __fmul_rn(kext[n], fld[n]));
                A[n * C + o] = a;
                ade[n] = a;
            }
        }
    }
    // dispersion orders 1..3 (materials with several poles): the same update
    // of each order's states from the same old field, in order
    // (engine_ext_lorentzmaterial.cpp:80-121 loop over o); the new states
    // stay in global memory and are subtracted after the node update
    if ((FEAT & FEAT_ADEX) && (flags & TF_ADEX_ALL)) {
        float* Ax = H ? g.AIx : g.AVx;
        float* Lx = H ? g.LIx : g.LVx;
#pragma unroll 1
        for (int k = 0; k < kExtraOrders; ++k) {
            if (!(flags & (TF_ADEX << k))) continue;
            const float4* ta = T.adex + ((long long)k * T.ntup + t) * TAB_ADE;
            const float4 a0 = __ldg(ta);
            const float4 a1 = __ldg(ta + 1);
            const float4 a2 = __ldg(ta + 2);
            const float kint[3] = {a0.x, a0.y, a0.z};
            const float kext[3] = {a0.w, a1.x, a1.y};
            const float klor[3] = {a1.z, a1.w, a2.x};
            float* As = Ax + (long long)k * 3 * C;
            const bool lor = (flags & (TF_LORX << k)) != 0;
#pragma unroll
            for (int n = 0; n < 3; ++n) {
                float a = As[n * C + o];
                float f = fld[n];
                if (lor) {
                    float* Ls = Lx + (long long)k * 3 * C;
                    const float l = __fadd_rn(Ls[n * C + o], __fmul_rn(klor[n], a));
                    Ls[n * C + o] = l;
                    f = __fsub_rn(f, l);
                }
                a = __fmul_rn(a, kint[n]);
                a = __fadd_rn(a, __fmul_rn(kext[n], f));
                As[n * C + o] = a;
            }
        }
    }
    if ((FEAT & FEAT_UPML) && (flags & TF_UPML)) {
        const float4 u0 = __ldg(&T.upml[TAB_UPML * t]);
        const float4 u1 = __ldg(&T.upml[TAB_UPML * t + 1]);
        const float4 u2 = __ldg(&T.upml[TAB_UPML * t + 2]);
        const float kp[3] = {u0.x, u0.y, u0.z};
        const float kfo[3] = {u0.w, u1.x, u1.y};
        const float kfn[3] = {u1.z, u1.w, u2.x};
#pragma unroll
        for (int n = 0; n < 3; ++n) {
            const float F = fsrc ? fsrc[n * fstride] : Fl[n * C + o];
            const float f = __fsub_rn(__fmul_rn(kp[n], fld[n]), __fmul_rn(kfo[n], F));
            const float Fn = __fadd_rn(__fmul_rn(F, c1[n]), __fmul_rn(c2[n], curl[n]));
            if (fwrite) Fl[n * C + o] = Fn;
            fld[n] = __fadd_rn(f, __fmul_rn(kfn[n], Fn));
        }
    } else {
#pragma unroll
        for (int n = 0; n < 3; ++n) fld[n] = __fadd_rn(__fmul_rn(fld[n], c1[n]), __fmul_rn(c2[n], curl[n]));
    }
    if ((FEAT & FEAT_ADE) && (flags & TF_ADE)) {
#pragma unroll
        for (int n = 0; n < 3; ++n) fld[n] = __fsub_rn(fld[n], ade[n]);
    }
    // V -= ADE of each further order, order by order (engine_ext_dispersive.cpp:76-132)
    if ((FEAT & FEAT_ADEX) && (flags & TF_ADEX_ALL)) {
        const float* Ax = H ? g.AIx : g.AVx;
#pragma unroll 1
        for (int k = 0; k < kExtraOrders; ++k) {
            if (!(flags & (TF_ADEX << k))) continue;
#pragma unroll
            for (int n = 0; n < 3; ++n) fld[n] = __fsub_rn(fld[n], Ax[(long long)k * 3 * C + n * C + o]);
        }
    }
    if (flags & TF_EXC) {
        const float4 e0 = __ldg(&T.exc[TAB_EXC * t]);
        const float4 e1 = __ldg(&T.exc[TAB_EXC * t + 1]);
        const float amp[3] = {e0.x, e0.y, e0.z};
        const int dly[3] = {__float_as_int(e1.x), __float_as_int(e1.y), __float_as_int(e1.z)};
        const float* sig = H ? g.sigC : g.sigV;
#pragma unroll
        for (int n = 0; n < 3; ++n)
            if (dly[n] >= 0) {
                const int k = exc_index(numTS, dly[n], g.sig_len, g.sig_period);
                fld[n] = __fadd_rn(fld[n], __fmul_rn(amp[n], sig[k]));
            }
    }
}

}  // namespace wipems
