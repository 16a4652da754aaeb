// Device side of the GB300 FDTD engine: the two fused half-step kernels,
// the probe / energy reductions and the timestep counter.
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
// result is bit-identical to the FP32 CPU engine.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace wipems {

// table entry flags (bits of the 7th float of the main entry)
constexpr uint32_t TF_UPML = 1u;
constexpr uint32_t TF_ADE = 2u;
constexpr uint32_t TF_LOR = 4u;
constexpr uint32_t TF_EXC = 8u;

// kernel feature bits (compile time)
constexpr int FEAT_UPML = 1;
constexpr int FEAT_ADE = 2;

struct DevGrid {
    int Nx, Ny, Nz;      // mesh lines
    int Nzp;             // padded z stride (multiple of 32)
    long long sx;        // x stride (Ny*Nzp)
    long long comp;      // component stride (Nx*Ny*Nzp)
    float* V;            // [3][comp]
    float* I;            // [3][comp]
    float* FV;           // UPML voltage flux [3][comp] or null
    float* FI;           // UPML current flux
    float* AV;           // ADE voltage state (order 1) [3][comp]
    float* LV;           // Lorentz voltage state
    float* AI;           // ADE current state
    float* LI;
    const void* idx;     // per-node tuple index (uint16 or uint32) [comp]
    const float4* tabE;  // [T][2] {vv0,vv1,vv2,vi0},{vi1,vi2,flags,-}
    const float4* tabH;  // [T][2] {ii0,ii1,ii2,iv0},{iv1,iv2,flags,-}
    const float4* tabEU; // [T][3] {vvp0..2,vvfo0},{vvfo1,vvfo2,vvfn0,vvfn1},{vvfn2,-,-,-}
    const float4* tabHU; // [T][3]
    const float4* tabEA; // [T][3] {vint0..2,vext0},{vext1,vext2,vlor0,vlor1},{vlor2,-,-,-}
    const float4* tabHA; // [T][3]
    const float4* tabEX; // [T][2] {amp0..2,-},{delay0..2 (int bits),-}
    const float4* tabHX; // [T][2]
    const float* sigV;   // excitation signals
    const float* sigC;
    int sig_len;
    int sig_period;      // 0 = none
    const int* d_ts;     // timestep counter (numTS)
    double* d_eacc;      // energy accumulators {sum V^2, sum I^2}
};

template <typename IdxT>
__device__ __forceinline__ uint32_t load_idx(const void* p, long long o) {
    return (uint32_t)__ldg(reinterpret_cast<const IdxT*>(p) + o);
}

__device__ __forceinline__ int exc_index(int numTS, int delay, int length, int period) {
    // engine_ext_excitation.cpp:44-53
    int exc_pos = numTS - delay;
    exc_pos *= (exc_pos > 0);
    int p = period > 0 ? period : numTS + 1;
    exc_pos %= p;
    exc_pos *= (exc_pos < length);
    return exc_pos;
}

// --------------------------------------------------------------- E half-step
// Block: 32 (z) x TY (y) threads, marching over x in [x0, x0+XC).
// Shared memory double buffer: 3 components x (TY+1) rows x 33 cols; row 0 is
// the y-1 halo, column 0 the z-1 halo.
template <typename IdxT, int FEAT>
__global__ void __launch_bounds__(256) k_volt(const DevGrid g, int ts_off, int XC) {
    extern __shared__ float smem[];
    const int TY = blockDim.y;
    const int tz = threadIdx.x, ty = threadIdx.y;
    const int z = blockIdx.x * 32 + tz;
    const int y = blockIdx.y * TY + ty;
    const int x0 = blockIdx.z * XC;
    const int x1 = min(x0 + XC, g.Nx);
    const bool valid = (z < g.Nz) && (y < g.Ny);
    const int rows = TY + 1;
    const int bufsz = 3 * rows * 33;
    const int numTS = *g.d_ts + ts_off;

    const long long yz = (long long)y * g.Nzp + z;
    const long long C = g.comp;
    float p1 = 0.f, p2 = 0.f;  // I1, I2 at x-1
    if (valid && x0 > 0) {
        long long o = (long long)(x0 - 1) * g.sx + yz;
        p1 = g.I[C + o];
        p2 = g.I[2 * C + o];
    }
    for (int x = x0; x < x1; ++x) {
        float* s = smem + ((x - x0) & 1) * bufsz;
        float* s0 = s;
        float* s1 = s + rows * 33;
        float* s2 = s + 2 * rows * 33;
        const long long o = (long long)x * g.sx + yz;
        float c0 = 0.f, c1 = 0.f, c2 = 0.f;
        if (valid) {
            c0 = g.I[o];
            c1 = g.I[C + o];
            c2 = g.I[2 * C + o];
        }
        const int si = (ty + 1) * 33 + tz + 1;
        s0[si] = c0;
        s1[si] = c1;
        s2[si] = c2;
        if (ty == 0 && y > 0 && z < g.Nz) {  // y-1 halo row: I0, I2
            long long oh = o - g.Nzp;
            s0[tz + 1] = g.I[oh];
            s2[tz + 1] = g.I[2 * C + oh];
        }
        if (tz == 0 && z > 0 && y < g.Ny) {  // z-1 halo column: I0, I1
            long long oh = o - 1;
            s0[(ty + 1) * 33] = g.I[oh];
            s1[(ty + 1) * 33] = g.I[C + oh];
        }
        __syncthreads();
        if (valid) {
            const float i2ym = (y > 0) ? s2[si - 33] : c2;
            const float i0ym = (y > 0) ? s0[si - 33] : c0;
            const float i1zm = (z > 0) ? s1[si - 1] : c1;
            const float i0zm = (z > 0) ? s0[si - 1] : c0;
            const float i2xm = (x > 0) ? p2 : c2;
            const float i1xm = (x > 0) ? p1 : c1;
            float curl[3];
            curl[0] = __fadd_rn(__fsub_rn(__fsub_rn(c2, i2ym), c1), i1zm);
            curl[1] = __fadd_rn(__fsub_rn(__fsub_rn(c0, i0zm), c2), i2xm);
            curl[2] = __fadd_rn(__fsub_rn(__fsub_rn(c1, i1xm), c0), i0ym);

            const uint32_t t = load_idx<IdxT>(g.idx, o);
            const float4 ta = __ldg(&g.tabE[2 * t]);
            const float4 tb = __ldg(&g.tabE[2 * t + 1]);
            const float vvc[3] = {ta.x, ta.y, ta.z};
            const float vic[3] = {ta.w, tb.x, tb.y};
            const uint32_t flags = __float_as_uint(tb.z);

            float v[3];
            v[0] = g.V[o];
            v[1] = g.V[C + o];
            v[2] = g.V[2 * C + o];

            // ADE pre-update with the old voltage (Lorentz extension, priority 0)
            float ade[3] = {0.f, 0.f, 0.f};
            if ((FEAT & FEAT_ADE) && (flags & TF_ADE)) {
                const float4 a0 = __ldg(&g.tabEA[3 * t]);
                const float4 a1 = __ldg(&g.tabEA[3 * t + 1]);
                const float4 a2 = __ldg(&g.tabEA[3 * t + 2]);
                const float vint[3] = {a0.x, a0.y, a0.z};
                const float vext[3] = {a0.w, a1.x, a1.y};
                const float vlor[3] = {a1.z, a1.w, a2.x};
                if (flags & TF_LOR) {
#pragma unroll
                    for (int n = 0; n < 3; ++n) {
                        float lor = g.LV[n * C + o];
                        float a = g.AV[n * C + o];
                        lor = __fadd_rn(lor, __fmul_rn(vlor[n], a));
                        a = __fmul_rn(a, vint[n]);
                        a = __fadd_rn(a, __fmul_rn(vext[n], __fsub_rn(v[n], lor)));
                        g.LV[n * C + o] = lor;
                        g.AV[n * C + o] = a;
                        ade[n] = a;
                    }
                } else {
#pragma unroll
                    for (int n = 0; n < 3; ++n) {
                        float a = g.AV[n * C + o];
                        a = __fmul_rn(a, vint[n]);
                        a = __fadd_rn(a, __fmul_rn(vext[n], v[n]));
                        g.AV[n * C + o] = a;
                        ade[n] = a;
                    }
                }
            }

            if ((FEAT & FEAT_UPML) && (flags & TF_UPML)) {
                const float4 u0 = __ldg(&g.tabEU[3 * t]);
                const float4 u1 = __ldg(&g.tabEU[3 * t + 1]);
                const float4 u2 = __ldg(&g.tabEU[3 * t + 2]);
                const float vvp[3] = {u0.x, u0.y, u0.z};
                const float vvfo[3] = {u0.w, u1.x, u1.y};
                const float vvfn[3] = {u1.z, u1.w, u2.x};
#pragma unroll
                for (int n = 0; n < 3; ++n) {
                    const float F = g.FV[n * C + o];
                    const float f = __fsub_rn(__fmul_rn(vvp[n], v[n]), __fmul_rn(vvfo[n], F));
                    const float Fn = __fadd_rn(__fmul_rn(F, vvc[n]), __fmul_rn(vic[n], curl[n]));
                    g.FV[n * C + o] = Fn;
                    v[n] = __fadd_rn(f, __fmul_rn(vvfn[n], Fn));
                }
            } else {
#pragma unroll
                for (int n = 0; n < 3; ++n)
                    v[n] = __fadd_rn(__fmul_rn(v[n], vvc[n]), __fmul_rn(vic[n], curl[n]));
            }
            if ((FEAT & FEAT_ADE) && (flags & TF_ADE)) {
#pragma unroll
                for (int n = 0; n < 3; ++n) v[n] = __fsub_rn(v[n], ade[n]);
            }
            if (flags & TF_EXC) {
                const float4 e0 = __ldg(&g.tabEX[2 * t]);
                const float4 e1 = __ldg(&g.tabEX[2 * t + 1]);
                const float amp[3] = {e0.x, e0.y, e0.z};
                const int dly[3] = {__float_as_int(e1.x), __float_as_int(e1.y), __float_as_int(e1.z)};
#pragma unroll
                for (int n = 0; n < 3; ++n)
                    if (dly[n] >= 0) {
                        const int k = exc_index(numTS, dly[n], g.sig_len, g.sig_period);
                        v[n] = __fadd_rn(v[n], __fmul_rn(amp[n], g.sigV[k]));
                    }
            }
            g.V[o] = v[0];
            g.V[C + o] = v[1];
            g.V[2 * C + o] = v[2];
        }
        p1 = c1;
        p2 = c2;
    }
}

// --------------------------------------------------------------- H half-step
// Same tiling; marching over x needs plane x+1 (registers) and the y+1 / z+1
// neighbours of plane x (shared memory: row TY is the y+1 halo, column 32
// the z+1 halo).
template <typename IdxT, int FEAT, bool ENERGY>
__global__ void __launch_bounds__(256) k_curr(const DevGrid g, int ts_off, int XC) {
    extern __shared__ float smem[];
    const int TY = blockDim.y;
    const int tz = threadIdx.x, ty = threadIdx.y;
    const int z = blockIdx.x * 32 + tz;
    const int y = blockIdx.y * TY + ty;
    const int x0 = blockIdx.z * XC;
    const int x1 = min(x0 + XC, g.Nx - 1);  // currents live on x < Nx-1
    const bool inplane = (z < g.Nz) && (y < g.Ny);
    const bool active = (z < g.Nz - 1) && (y < g.Ny - 1);
    const int rows = TY + 1;
    const int bufsz = 3 * rows * 33;
    const int numTS = *g.d_ts + ts_off;

    const long long yz = (long long)y * g.Nzp + z;
    const long long C = g.comp;
    double esum = 0.0, hsum = 0.0;
    float c0 = 0.f, c1 = 0.f, c2 = 0.f;  // V at plane x
    if (inplane && x0 < x1) {
        long long o = (long long)x0 * g.sx + yz;
        c0 = g.V[o];
        c1 = g.V[C + o];
        c2 = g.V[2 * C + o];
    }
    for (int x = x0; x < x1; ++x) {
        float* s = smem + ((x - x0) & 1) * bufsz;
        float* s0 = s;
        float* s1 = s + rows * 33;
        float* s2 = s + 2 * rows * 33;
        const long long o = (long long)x * g.sx + yz;
        float n1 = 0.f, n2 = 0.f, n0 = 0.f;  // V at plane x+1
        if (inplane) {
            const long long on = o + g.sx;
            n0 = g.V[on];
            n1 = g.V[C + on];
            n2 = g.V[2 * C + on];
        }
        const int si = ty * 33 + tz;
        s0[si] = c0;
        s1[si] = c1;
        s2[si] = c2;
        if (ty == TY - 1 && y + 1 < g.Ny && z < g.Nz) {  // y+1 halo row: V0, V2
            long long oh = o + g.Nzp;
            s0[TY * 33 + tz] = g.V[oh];
            s2[TY * 33 + tz] = g.V[2 * C + oh];
        }
        if (tz == 31 && z + 1 < g.Nz && y < g.Ny) {  // z+1 halo column: V0, V1
            long long oh = o + 1;
            s0[ty * 33 + 32] = g.V[oh];
            s1[ty * 33 + 32] = g.V[C + oh];
        }
        __syncthreads();
        if (active) {
            const float v2yp = s2[si + 33];
            const float v0yp = s0[si + 33];
            const float v1zp = s1[si + 1];
            const float v0zp = s0[si + 1];
            float curl[3];
            curl[0] = __fadd_rn(__fsub_rn(__fsub_rn(c2, v2yp), c1), v1zp);
            curl[1] = __fadd_rn(__fsub_rn(__fsub_rn(c0, v0zp), c2), n2);
            curl[2] = __fadd_rn(__fsub_rn(__fsub_rn(c1, n1), c0), v0yp);

            const uint32_t t = load_idx<IdxT>(g.idx, o);
            const float4 ta = __ldg(&g.tabH[2 * t]);
            const float4 tb = __ldg(&g.tabH[2 * t + 1]);
            const float iic[3] = {ta.x, ta.y, ta.z};
            const float ivc[3] = {ta.w, tb.x, tb.y};
            const uint32_t flags = __float_as_uint(tb.z);

            float cu[3];
            cu[0] = g.I[o];
            cu[1] = g.I[C + o];
            cu[2] = g.I[2 * C + o];

            float ade[3] = {0.f, 0.f, 0.f};
            if ((FEAT & FEAT_ADE) && (flags & TF_ADE)) {
                const float4 a0 = __ldg(&g.tabHA[3 * t]);
                const float4 a1 = __ldg(&g.tabHA[3 * t + 1]);
                const float4 a2 = __ldg(&g.tabHA[3 * t + 2]);
                const float iint[3] = {a0.x, a0.y, a0.z};
                const float iext[3] = {a0.w, a1.x, a1.y};
                const float ilor[3] = {a1.z, a1.w, a2.x};
                if (flags & TF_LOR) {
#pragma unroll
                    for (int n = 0; n < 3; ++n) {
                        float lor = g.LI[n * C + o];
                        float a = g.AI[n * C + o];
                        lor = __fadd_rn(lor, __fmul_rn(ilor[n], a));
                        a = __fmul_rn(a, iint[n]);
                        a = __fadd_rn(a, __fmul_rn(iext[n], __fsub_rn(cu[n], lor)));
                        g.LI[n * C + o] = lor;
                        g.AI[n * C + o] = a;
                        ade[n] = a;
                    }
                } else {
#pragma unroll
                    for (int n = 0; n < 3; ++n) {
                        float a = g.AI[n * C + o];
                        a = __fmul_rn(a, iint[n]);
                        a = __fadd_rn(a, __fmul_rn(iext[n], cu[n]));
                        g.AI[n * C + o] = a;
                        ade[n] = a;
                    }
                }
            }
            if ((FEAT & FEAT_UPML) && (flags & TF_UPML)) {
                const float4 u0 = __ldg(&g.tabHU[3 * t]);
                const float4 u1 = __ldg(&g.tabHU[3 * t + 1]);
                const float4 u2 = __ldg(&g.tabHU[3 * t + 2]);
                const float iip[3] = {u0.x, u0.y, u0.z};
                const float iifo[3] = {u0.w, u1.x, u1.y};
                const float iifn[3] = {u1.z, u1.w, u2.x};
#pragma unroll
                for (int n = 0; n < 3; ++n) {
                    const float F = g.FI[n * C + o];
                    const float f = __fsub_rn(__fmul_rn(iip[n], cu[n]), __fmul_rn(iifo[n], F));
                    const float Fn = __fadd_rn(__fmul_rn(F, iic[n]), __fmul_rn(ivc[n], curl[n]));
                    g.FI[n * C + o] = Fn;
                    cu[n] = __fadd_rn(f, __fmul_rn(iifn[n], Fn));
                }
            } else {
#pragma unroll
                for (int n = 0; n < 3; ++n)
                    cu[n] = __fadd_rn(__fmul_rn(cu[n], iic[n]), __fmul_rn(ivc[n], curl[n]));
            }
            if ((FEAT & FEAT_ADE) && (flags & TF_ADE)) {
#pragma unroll
                for (int n = 0; n < 3; ++n) cu[n] = __fsub_rn(cu[n], ade[n]);
            }
            if (flags & TF_EXC) {
                const float4 e0 = __ldg(&g.tabHX[2 * t]);
                const float4 e1 = __ldg(&g.tabHX[2 * t + 1]);
                const float amp[3] = {e0.x, e0.y, e0.z};
                const int dly[3] = {__float_as_int(e1.x), __float_as_int(e1.y), __float_as_int(e1.z)};
#pragma unroll
                for (int n = 0; n < 3; ++n)
                    if (dly[n] >= 0) {
                        const int k = exc_index(numTS, dly[n], g.sig_len, g.sig_period);
                        cu[n] = __fadd_rn(cu[n], __fmul_rn(amp[n], g.sigC[k]));
                    }
            }
            g.I[o] = cu[0];
            g.I[C + o] = cu[1];
            g.I[2 * C + o] = cu[2];
            if (ENERGY) {
                // Engine_Interface_FDTD::CalcFastEnergy terms (float products)
                esum += (double)__fmul_rn(c0, c0) + (double)__fmul_rn(c1, c1) + (double)__fmul_rn(c2, c2);
                hsum += (double)__fmul_rn(cu[0], cu[0]) + (double)__fmul_rn(cu[1], cu[1]) +
                        (double)__fmul_rn(cu[2], cu[2]);
            }
        }
        c0 = n0;
        c1 = n1;
        c2 = n2;
    }
    if (ENERGY) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            esum += __shfl_down_sync(0xffffffffu, esum, off);
            hsum += __shfl_down_sync(0xffffffffu, hsum, off);
        }
        if (tz == 0 && (esum != 0.0 || hsum != 0.0)) {
            atomicAdd(&g.d_eacc[0], esum);
            atomicAdd(&g.d_eacc[1], hsum);
        }
    }
}

// ---------------------------------------------------------- probes / counter
struct ProbeEntry {
    uint32_t off;   // linear offset within the component (padded layout)
    int8_t comp;    // 0..2
    int8_t sign;    // +1 / -1
    int8_t field;   // 0 = voltage, 1 = current
    int8_t pad;
};

struct ProbeSet {
    const ProbeEntry* entries;  // all probes' entries, concatenated
    const int* first;           // [nprobe+1] entry ranges
    const double* weight;       // [nprobe]
    int nprobe;
    int row_doubles;            // doubles per record row (2 + nprobe)
    double* ring;               // [cap][row_doubles]: ts, energy, values...
    int cap;
    int* d_nsamp;               // samples written
    int* d_err;                 // error word (ring overflow, non-finite)
};

// Advances numTS by adv (Engine::IterateTS ++numTS) and, when sample is set,
// records one probe/energy sample row (ProcessIntegral::Process).
__global__ void k_advance_sample(int* d_ts, int adv, int sample, ProbeSet ps, const DevGrid g,
                                 int energy_valid, double eps0, double mue0) {
    __shared__ int s_ts, s_row;
    if (threadIdx.x == 0) {
        int ts = *d_ts + adv;
        if (adv) *d_ts = ts;
        s_ts = ts;
        s_row = -1;
        if (sample) {
            int row = *ps.d_nsamp;
            if (row < ps.cap) {
                s_row = row;
                *ps.d_nsamp = row + 1;
            } else {
                atomicOr(ps.d_err, 1);
            }
        }
    }
    __syncthreads();
    if (!sample || s_row < 0) return;
    double* rec = ps.ring + (long long)s_row * ps.row_doubles;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nwarps = blockDim.x >> 5;
    for (int p = warp; p < ps.nprobe; p += nwarps) {
        double acc = 0.0;
        for (int e = ps.first[p] + lane; e < ps.first[p + 1]; e += 32) {
            const ProbeEntry pe = ps.entries[e];
            const float* f = pe.field ? g.I : g.V;
            const float val = f[(long long)pe.comp * g.comp + pe.off];
            acc += pe.sign > 0 ? (double)val : -(double)val;
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
        if (lane == 0) rec[2 + p] = acc * ps.weight[p];
    }
    if (threadIdx.x == 0) {
        rec[0] = (double)s_ts;
        if (energy_valid) {
            double e = eps0 * g.d_eacc[0] + mue0 * g.d_eacc[1];
            if (!isfinite(e)) atomicOr(ps.d_err, 2);
            rec[1] = e;
        } else {
            rec[1] = -1.0;
        }
        g.d_eacc[0] = 0.0;
        g.d_eacc[1] = 0.0;
    }
}

// Full-grid energy (CalcFastEnergy) on demand.
__global__ void k_energy(const DevGrid g, double* out) {
    double es = 0.0, hs = 0.0;
    const long long nyz = (long long)(g.Ny - 1) * (g.Nz - 1);
    const long long total = (long long)(g.Nx - 1) * nyz;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i / nyz);
        const long long r = i - (long long)x * nyz;
        const int y = (int)(r / (g.Nz - 1));
        const int z = (int)(r - (long long)y * (g.Nz - 1));
        const long long o = (long long)x * g.sx + (long long)y * g.Nzp + z;
#pragma unroll
        for (int n = 0; n < 3; ++n) {
            const float v = g.V[n * g.comp + o];
            const float c = g.I[n * g.comp + o];
            es += (double)__fmul_rn(v, v);
            hs += (double)__fmul_rn(c, c);
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        es += __shfl_down_sync(0xffffffffu, es, off);
        hs += __shfl_down_sync(0xffffffffu, hs, off);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&out[0], es);
        atomicAdd(&out[1], hs);
    }
}

}  // namespace wipems
