// TMA-pipelined half-step kernels (sm_100+/sm_103a).
//
// Same per-node arithmetic as kernels.cuh (k_volt / k_curr, which cite the
// reference); what changes is how data reaches the SM.  A block owns a tile
// of TZ = 32*ZW (z) x TY (y) nodes -- each thread updates ZW consecutive z
// nodes with vector shared/global accesses -- and marches over an x-chunk.  Each x-plane of the
// tile -- the three field components of both halves with the one-node halo
// the curl needs, the tuple index and, in UPML tiles, the flux -- is fetched
// by one thread with cp.async.bulk.tensor (TMA) into a ring of STAGES
// shared-memory buffers, STAGES-1 planes ahead of the plane being computed,
// completion tracked by one mbarrier per stage.  Compute threads read only
// shared memory and registers; results are stored straight to global.
//
// TMA boxes (innermost first; the fourth dimension spans the 3 components):
//   E kernel: I halo box {TZ+4, TY+1, 1, 3} at (z0-4, y0-1, x)  (z-1, y-1 halo)
//             V own box  {TZ, TY, 1, 3}     at (z0, y0, x)
//             idx box    {TZ, TY, 1}        at (z0, y0, x)
//             V-flux box {TZ, TY, 1, 3}     (UPML tiles only)
//   H kernel: V halo box {TZ+4, TY+1, 1, 3} at (z0, y0, x)      (z+1, y+1 halo)
//             I own box  {TZ, TY, 1, 3}, idx box, I-flux box
// The innermost start coordinate is always a multiple of 4 floats (16 B);
// out-of-range parts of a box (z<0, y<0, beyond the grid) read zeros.
//
// Every wait on an mbarrier is bounded by a clock budget; on expiry the block
// raises bit 4 of the engine's error word, stops computing (the whole block
// leaves the plane loop together via __syncthreads_or), waits -- again with
// a budget -- for the copies it has in flight, and returns.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include "kernels.cuh"

namespace wipems {

constexpr int TMA_MAX_STAGES = 8;
constexpr int TMA_TY = 8;
constexpr unsigned long long TMA_WAIT_CYCLES = 4000000000ull;  // ~2 s at 2 GHz

struct TmaMaps {
    CUtensorMap I_halo, I_own, V_halo, V_own, FV_own, FI_own, idx;
};

// geometry of the UPML slabs: a node is in a slab iff one coordinate is
// outside [lo, hi] of its axis (empty slab set: lo = 0, hi = N-1); ne[] is
// the extent of the voltage update (N, or N-1 where the last line of that
// axis holds only PEC edges and no extension state: its voltages stay 0)
struct TileInfo {
    int lo[3], hi[3];
    int ne[3];
    int* d_err;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait: false when the clock budget ran out
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = clock64();
    while (!mbar_try_wait(bar, parity)) {
        if (clock64() - t0 > TMA_WAIT_CYCLES) return false;
    }
    return true;
}
__device__ __forceinline__ void fence_barrier_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void tma_4d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1, int c2,
                                       int c3) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void tma_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1, int c2) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
        : "memory");
}

// stage layout (floats, every buffer 128-byte aligned)
template <typename IdxT, bool UPML, int ZW>
struct StageLayout {
    static constexpr int TZ = 32 * ZW;
    static constexpr int HW = TZ + 4;                            // halo box row width
    static constexpr int HALO = 3 * (TMA_TY + 1) * HW;           // halo box, 3 components
    static constexpr int HALO_A = (HALO + 31) / 32 * 32;
    static constexpr int OWN = 3 * TMA_TY * TZ;                  // own box, 3 components
    static constexpr int IDX = TMA_TY * TZ * (int)sizeof(IdxT) / 4;
    static constexpr int IDX_A = (IDX + 31) / 32 * 32;
    static constexpr int FLUX = UPML ? OWN : 0;
    static constexpr int STAGE = HALO_A + OWN + IDX_A + FLUX;    // floats
    static constexpr int HALO_BYTES = HALO * 4;
    static constexpr int OWN_BYTES = OWN * 4;
    static constexpr int IDX_BYTES = TMA_TY * TZ * (int)sizeof(IdxT);
    // + barriers + slack to align the dynamic shared memory base to 128 bytes
    static size_t smem(int stages) { return (size_t)STAGE * 4 * stages + 8 * TMA_MAX_STAGES + 128; }
};

__device__ __forceinline__ bool tile_has_upml(const TileInfo& ti, int x, int y0, int y1, int z0, int z1) {
    // any node of [z0,z1] x [y0,y1] at plane x outside the inner box
    if (x < ti.lo[0] || x > ti.hi[0]) return true;
    if (y0 < ti.lo[1] || y1 > ti.hi[1]) return true;
    if (z0 < ti.lo[2] || z1 > ti.hi[2]) return true;
    return false;
}

__device__ __forceinline__ void kahan_add(float& s, float& c, float x) {
    const float y = __fsub_rn(x, c);
    const float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);
    s = t;
}

// One voltage node: ADE pre-update (old V), main update with the UPML flux
// swap fused, ADE apply, excitation -- the hook order of Engine::IterateTS.
// F is the node's old UPML flux (read by the caller from shared or global
// memory) and is only used for UPML nodes.
template <int FEAT>
__device__ __forceinline__ void volt_node(const DevGrid& g, float v[3], const float curl[3], uint32_t t,
                                          long long o, int numTS, const float* fsrc, int fstride) {
    const float4 ta = __ldg(&g.tabE[2 * t]);
    const float4 tb = __ldg(&g.tabE[2 * t + 1]);
    const float vvc[3] = {ta.x, ta.y, ta.z};
    const float vic[3] = {ta.w, tb.x, tb.y};
    const uint32_t flags = __float_as_uint(tb.z);
    const long long C = g.comp;
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
            const float F = fsrc ? fsrc[n * fstride] : g.FV[n * C + o];
            const float f = __fsub_rn(__fmul_rn(vvp[n], v[n]), __fmul_rn(vvfo[n], F));
            const float Fn = __fadd_rn(__fmul_rn(F, vvc[n]), __fmul_rn(vic[n], curl[n]));
            g.FV[n * C + o] = Fn;
            v[n] = __fadd_rn(f, __fmul_rn(vvfn[n], Fn));
        }
    } else {
#pragma unroll
        for (int n = 0; n < 3; ++n) v[n] = __fadd_rn(__fmul_rn(v[n], vvc[n]), __fmul_rn(vic[n], curl[n]));
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
}

// One current node (mirror of volt_node for the H half-step).
template <int FEAT>
__device__ __forceinline__ void curr_node(const DevGrid& g, float cu[3], const float curl[3], uint32_t t,
                                          long long o, int numTS, const float* fsrc, int fstride) {
    const float4 ta = __ldg(&g.tabH[2 * t]);
    const float4 tb = __ldg(&g.tabH[2 * t + 1]);
    const float iic[3] = {ta.x, ta.y, ta.z};
    const float ivc[3] = {ta.w, tb.x, tb.y};
    const uint32_t flags = __float_as_uint(tb.z);
    const long long C = g.comp;
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
            const float F = fsrc ? fsrc[n * fstride] : g.FI[n * C + o];
            const float f = __fsub_rn(__fmul_rn(iip[n], cu[n]), __fmul_rn(iifo[n], F));
            const float Fn = __fadd_rn(__fmul_rn(F, iic[n]), __fmul_rn(ivc[n], curl[n]));
            g.FI[n * C + o] = Fn;
            cu[n] = __fadd_rn(f, __fmul_rn(iifn[n], Fn));
        }
    } else {
#pragma unroll
        for (int n = 0; n < 3; ++n) cu[n] = __fadd_rn(__fmul_rn(cu[n], iic[n]), __fmul_rn(ivc[n], curl[n]));
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
}

template <int ZW>
struct VecT;
template <>
struct VecT<1> {
    typedef float F;
    __device__ static float get(const float& v, int) { return v; }
};
template <>
struct VecT<2> {
    typedef float2 F;
    __device__ static float get(const float2& v, int k) { return k ? v.y : v.x; }
};

// ------------------------------------------------------------- E half-step
template <typename IdxT, int FEAT, int ZW>
__global__ void __launch_bounds__(TMA_TY * 32) k_volt_tma(const DevGrid g, const __grid_constant__ TmaMaps m,
                                                          const TileInfo ti, int ts_off, int XC, int STAGES) {
    constexpr bool UPML = (FEAT & FEAT_UPML) != 0;
    using L = StageLayout<IdxT, UPML, ZW>;
    using V = VecT<ZW>;
    typedef typename V::F VF;
    constexpr int TZ = L::TZ, HW = L::HW;
    extern __shared__ __align__(128) float smem_raw[];
    float* smem = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~(uintptr_t)127);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + (size_t)L::STAGE * STAGES);
    const int tz = threadIdx.x, ty = threadIdx.y;
    const int tid = ty * 32 + tz;
    const int z0 = blockIdx.x * TZ, y0 = blockIdx.y * TMA_TY;
    const int zt = ZW * tz;                 // first z of the thread within the tile
    const int z = z0 + zt, y = y0 + ty;
    const int x0 = blockIdx.z * XC;
    const int x1 = min(x0 + XC, ti.ne[0]);
    const int nplanes = x1 - x0;
    const bool rowok = y < ti.ne[1];
    const int nzv = min(ZW, ti.ne[2] - z);  // valid nodes of this thread
    const bool valid = rowok && nzv > 0;
    const int numTS = *g.d_ts + ts_off;
    const long long C = g.comp;
    const int zl = min(z0 + TZ - 1, g.Nz - 1), yl = min(y0 + TMA_TY - 1, g.Ny - 1);

    if (tid == 0) {
        for (int s = 0; s < STAGES; ++s) mbar_init(&bars[s], 1);
        fence_barrier_init();
    }
    __syncthreads();

    auto issue = [&](int r) {  // thread 0: plane x0+r into stage r % STAGES
        const int s = r % STAGES;
        const int x = x0 + r;
        float* st = smem + (size_t)s * L::STAGE;
        const bool up = UPML && tile_has_upml(ti, x, y0, yl, z0, zl);
        const uint32_t bytes = L::HALO_BYTES + L::OWN_BYTES + L::IDX_BYTES + (up ? L::OWN_BYTES : 0);
        mbar_expect_tx(&bars[s], bytes);
        tma_4d(st, &m.I_halo, &bars[s], z0 - 4, y0 - 1, x, 0);
        tma_4d(st + L::HALO_A, &m.V_own, &bars[s], z0, y0, x, 0);
        tma_3d(st + L::HALO_A + L::OWN, &m.idx, &bars[s], z0, y0, x);
        if (up) tma_4d(st + L::HALO_A + L::OWN + L::IDX_A, &m.FV_own, &bars[s], z0, y0, x, 0);
    };

    int issued = 0;
    if (tid == 0) {
        for (; issued < min(STAGES - 1, nplanes); ++issued) issue(issued);
    }
    VF p1 = VF(), p2 = VF();  // I1, I2 at x-1
    const long long yz = (long long)y * g.Nzp + z;
    if (valid && x0 > 0) {
        const long long o = (long long)(x0 - 1) * g.sx + yz;
        p1 = *reinterpret_cast<const VF*>(g.I + C + o);
        p2 = *reinterpret_cast<const VF*>(g.I + 2 * C + o);
    }
    float* Vp = g.V + (long long)x0 * g.sx + yz;  // node (x0, y, z), advanced by sx per plane
    bool aborted = false;
    int r = 0;
    for (; r < nplanes; ++r, Vp += g.sx) {
        if (tid == 0 && issued < nplanes && issued == r + STAGES - 1) {
            fence_proxy_async();
            issue(issued);
            ++issued;
        }
        const int s = r % STAGES;
        const bool ok = mbar_wait(&bars[s], (uint32_t)((r / STAGES) & 1));
        const int x = x0 + r;
        const float* st = smem + (size_t)s * L::STAGE;
        VF c1v = VF(), c2v = VF();
        if (ok && valid) {
            const int hi = (ty + 1) * HW + 4 + zt;  // own position in the halo box
            const float* sI0 = st;
            const float* sI1 = st + (TMA_TY + 1) * HW;
            const float* sI2 = st + 2 * (TMA_TY + 1) * HW;
            const VF c0v = *reinterpret_cast<const VF*>(sI0 + hi);
            c1v = *reinterpret_cast<const VF*>(sI1 + hi);
            c2v = *reinterpret_cast<const VF*>(sI2 + hi);
            const VF i2ymv = *reinterpret_cast<const VF*>(sI2 + hi - HW);
            const VF i0ymv = *reinterpret_cast<const VF*>(sI0 + hi - HW);
            const float i1zm0 = sI1[hi - 1];
            const float i0zm0 = sI0[hi - 1];
            const int oi = ty * TZ + zt;
            const float* sV = st + L::HALO_A;
            const IdxT* sIdx = reinterpret_cast<const IdxT*>(st + L::HALO_A + L::OWN);
            const bool up = UPML && tile_has_upml(ti, x, y0, yl, z0, zl);
            const float* sF = up ? st + L::HALO_A + L::OWN + L::IDX_A : nullptr;
            const VF v0v = *reinterpret_cast<const VF*>(sV + oi);
            const VF v1v = *reinterpret_cast<const VF*>(sV + TMA_TY * TZ + oi);
            const VF v2v = *reinterpret_cast<const VF*>(sV + 2 * TMA_TY * TZ + oi);
            float outv[3][ZW];
#pragma unroll
            for (int k = 0; k < ZW; ++k) {
                const float c0 = V::get(c0v, k), c1 = V::get(c1v, k), c2 = V::get(c2v, k);
                const float i2ym = (y > 0) ? V::get(i2ymv, k) : c2;
                const float i0ym = (y > 0) ? V::get(i0ymv, k) : c0;
                const float i1zm = (k > 0) ? V::get(c1v, k - 1) : ((z > 0) ? i1zm0 : c1);
                const float i0zm = (k > 0) ? V::get(c0v, k - 1) : ((z > 0) ? i0zm0 : c0);
                const float i2xm = (x > 0) ? V::get(p2, k) : c2;
                const float i1xm = (x > 0) ? V::get(p1, k) : c1;
                float curl[3];
                curl[0] = __fadd_rn(__fsub_rn(__fsub_rn(c2, i2ym), c1), i1zm);
                curl[1] = __fadd_rn(__fsub_rn(__fsub_rn(c0, i0zm), c2), i2xm);
                curl[2] = __fadd_rn(__fsub_rn(__fsub_rn(c1, i1xm), c0), i0ym);
                float v[3] = {V::get(v0v, k), V::get(v1v, k), V::get(v2v, k)};
                if (k < nzv) {
                    const uint32_t t = (uint32_t)sIdx[oi + k];
                    const long long o = (long long)x * g.sx + yz + k;
                    volt_node<FEAT>(g, v, curl, t, o, numTS, sF ? sF + oi + k : nullptr, TMA_TY * TZ);
                }
                outv[0][k] = v[0];
                outv[1][k] = v[1];
                outv[2][k] = v[2];
            }
            if (nzv == ZW) {
#pragma unroll
                for (int n = 0; n < 3; ++n) {
                    VF w;
                    if constexpr (ZW == 2) w = make_float2(outv[n][0], outv[n][1]);
                    else w = outv[n][0];
                    *reinterpret_cast<VF*>(Vp + n * C) = w;
                }
            } else {
                for (int k = 0; k < nzv; ++k)
#pragma unroll
                    for (int n = 0; n < 3; ++n) Vp[n * C + k] = outv[n][k];
            }
        }
        p1 = c1v;
        p2 = c2v;
        if (__syncthreads_or(!ok)) {
            aborted = true;
            break;
        }
    }
    if (aborted && tid == 0) {
        atomicOr(ti.d_err, 4);
        // wait (bounded) for the copies this block still has in flight
        for (int q = r; q < issued; ++q) mbar_wait(&bars[q % STAGES], (uint32_t)((q / STAGES) & 1));
    }
}

// ------------------------------------------------------------- H half-step
template <typename IdxT, int FEAT, bool ENERGY, int ZW>
__global__ void __launch_bounds__(TMA_TY * 32) k_curr_tma(const DevGrid g, const __grid_constant__ TmaMaps m,
                                                          const TileInfo ti, int ts_off, int XC, int STAGES) {
    constexpr bool UPML = (FEAT & FEAT_UPML) != 0;
    using L = StageLayout<IdxT, UPML, ZW>;
    using V = VecT<ZW>;
    typedef typename V::F VF;
    constexpr int TZ = L::TZ, HW = L::HW;
    extern __shared__ __align__(128) float smem_raw[];
    float* smem = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~(uintptr_t)127);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + (size_t)L::STAGE * STAGES);
    const int tz = threadIdx.x, ty = threadIdx.y;
    const int tid = ty * 32 + tz;
    const int z0 = blockIdx.x * TZ, y0 = blockIdx.y * TMA_TY;
    const int zt = ZW * tz;
    const int z = z0 + zt, y = y0 + ty;
    const int x0 = blockIdx.z * XC;
    const int x1 = min(x0 + XC, g.Nx - 1);
    const int nplanes = x1 - x0;      // planes updated
    const int nload = nplanes + 1;    // plane x1 is read as the x+1 neighbour
    const int nzv = min(ZW, g.Nz - 1 - z);
    const bool active = (y < g.Ny - 1) && nzv > 0;
    const int numTS = *g.d_ts + ts_off;
    const long long C = g.comp;
    const int zl = min(z0 + TZ - 1, g.Nz - 1), yl = min(y0 + TMA_TY - 1, g.Ny - 1);

    if (tid == 0) {
        for (int s = 0; s < STAGES; ++s) mbar_init(&bars[s], 1);
        fence_barrier_init();
    }
    __syncthreads();

    auto issue = [&](int r) {
        const int s = r % STAGES;
        const int x = x0 + r;
        float* st = smem + (size_t)s * L::STAGE;
        const bool upd = r < nplanes;  // plane x1 only contributes V
        const bool up = UPML && upd && tile_has_upml(ti, x, y0, yl, z0, zl);
        const uint32_t bytes =
            L::HALO_BYTES + (upd ? L::OWN_BYTES + L::IDX_BYTES : 0) + (up ? L::OWN_BYTES : 0);
        mbar_expect_tx(&bars[s], bytes);
        tma_4d(st, &m.V_halo, &bars[s], z0, y0, x, 0);
        if (upd) {
            tma_4d(st + L::HALO_A, &m.I_own, &bars[s], z0, y0, x, 0);
            tma_3d(st + L::HALO_A + L::OWN, &m.idx, &bars[s], z0, y0, x);
        }
        if (up) tma_4d(st + L::HALO_A + L::OWN + L::IDX_A, &m.FI_own, &bars[s], z0, y0, x, 0);
    };

    int issued = 0;
    if (nplanes > 0 && tid == 0) {
        for (; issued < min(STAGES - 1, nload); ++issued) issue(issued);
    }
    float es = 0.f, ec = 0.f, hs = 0.f, hc = 0.f;  // Kahan sums of V^2 and I^2
    const long long yz = (long long)y * g.Nzp + z;
    float* Ip = g.I + (long long)x0 * g.sx + yz;
    bool aborted = false;
    int r = 0;
    for (; r < nplanes; ++r, Ip += g.sx) {
        if (tid == 0 && issued < nload && issued == r + STAGES - 1) {
            fence_proxy_async();
            issue(issued);
            ++issued;
        }
        const int s = r % STAGES;
        const int sn = (r + 1) % STAGES;
        bool ok = mbar_wait(&bars[s], (uint32_t)((r / STAGES) & 1));
        ok = ok && mbar_wait(&bars[sn], (uint32_t)(((r + 1) / STAGES) & 1));
        const int x = x0 + r;
        if (ok && active) {
            const float* st = smem + (size_t)s * L::STAGE;
            const float* stn = smem + (size_t)sn * L::STAGE;
            const float* sV0 = st;
            const float* sV1 = st + (TMA_TY + 1) * HW;
            const float* sV2 = st + 2 * (TMA_TY + 1) * HW;
            const int hi = ty * HW + zt;
            const VF c0v = *reinterpret_cast<const VF*>(sV0 + hi);
            const VF c1v = *reinterpret_cast<const VF*>(sV1 + hi);
            const VF c2v = *reinterpret_cast<const VF*>(sV2 + hi);
            const VF v2ypv = *reinterpret_cast<const VF*>(sV2 + hi + HW);
            const VF v0ypv = *reinterpret_cast<const VF*>(sV0 + hi + HW);
            const float v1zpL = sV1[hi + ZW];
            const float v0zpL = sV0[hi + ZW];
            const VF n1v = *reinterpret_cast<const VF*>(stn + (TMA_TY + 1) * HW + hi);
            const VF n2v = *reinterpret_cast<const VF*>(stn + 2 * (TMA_TY + 1) * HW + hi);
            const float* sI = st + L::HALO_A;
            const IdxT* sIdx = reinterpret_cast<const IdxT*>(st + L::HALO_A + L::OWN);
            const bool up = UPML && tile_has_upml(ti, x, y0, yl, z0, zl);
            const float* sF = up ? st + L::HALO_A + L::OWN + L::IDX_A : nullptr;
            const int oi = ty * TZ + zt;
            const VF i0v = *reinterpret_cast<const VF*>(sI + oi);
            const VF i1v = *reinterpret_cast<const VF*>(sI + TMA_TY * TZ + oi);
            const VF i2v = *reinterpret_cast<const VF*>(sI + 2 * TMA_TY * TZ + oi);
            float outc[3][ZW];
#pragma unroll
            for (int k = 0; k < ZW; ++k) {
                const float c0 = V::get(c0v, k), c1 = V::get(c1v, k), c2 = V::get(c2v, k);
                const float v1zp = (k + 1 < ZW) ? V::get(c1v, k + 1) : v1zpL;
                const float v0zp = (k + 1 < ZW) ? V::get(c0v, k + 1) : v0zpL;
                float curl[3];
                curl[0] = __fadd_rn(__fsub_rn(__fsub_rn(c2, V::get(v2ypv, k)), c1), v1zp);
                curl[1] = __fadd_rn(__fsub_rn(__fsub_rn(c0, v0zp), c2), V::get(n2v, k));
                curl[2] = __fadd_rn(__fsub_rn(__fsub_rn(c1, V::get(n1v, k)), c0), V::get(v0ypv, k));
                float cu[3] = {V::get(i0v, k), V::get(i1v, k), V::get(i2v, k)};
                if (k < nzv) {
                    const uint32_t t = (uint32_t)sIdx[oi + k];
                    const long long o = (long long)x * g.sx + yz + k;
                    curr_node<FEAT>(g, cu, curl, t, o, numTS, sF ? sF + oi + k : nullptr, TMA_TY * TZ);
                    if (ENERGY) {
                        kahan_add(es, ec, __fmul_rn(c0, c0));
                        kahan_add(es, ec, __fmul_rn(c1, c1));
                        kahan_add(es, ec, __fmul_rn(c2, c2));
                        kahan_add(hs, hc, __fmul_rn(cu[0], cu[0]));
                        kahan_add(hs, hc, __fmul_rn(cu[1], cu[1]));
                        kahan_add(hs, hc, __fmul_rn(cu[2], cu[2]));
                    }
                }
                outc[0][k] = cu[0];
                outc[1][k] = cu[1];
                outc[2][k] = cu[2];
            }
            if (nzv == ZW) {
#pragma unroll
                for (int n = 0; n < 3; ++n) {
                    VF w;
                    if constexpr (ZW == 2) w = make_float2(outc[n][0], outc[n][1]);
                    else w = outc[n][0];
                    *reinterpret_cast<VF*>(Ip + n * C) = w;
                }
            } else {
                for (int k = 0; k < nzv; ++k)
#pragma unroll
                    for (int n = 0; n < 3; ++n) Ip[n * C + k] = outc[n][k];
            }
        }
        if (__syncthreads_or(!ok)) {
            aborted = true;
            break;
        }
    }
    if (aborted && tid == 0) {
        atomicOr(ti.d_err, 4);
        for (int q = r; q < issued; ++q) mbar_wait(&bars[q % STAGES], (uint32_t)((q / STAGES) & 1));
    }
    if (ENERGY) {
        double esum = (double)es + (double)(-ec), hsum = (double)hs + (double)(-hc);
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

}  // namespace wipems
