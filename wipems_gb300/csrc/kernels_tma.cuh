// TMA-pipelined half-step kernels (sm_100+/sm_103a).
//
// Same per-node arithmetic as the direct kernels (node.cuh, which cites the
// reference); what changes is how data reaches the SM.  A block owns a tile
// of 32 (z) x TY (y) nodes and marches over an x-chunk.  Each x-plane of the
// tile -- the three components of both fields with the one-node halo the
// curl needs, the tuple index and, in UPML tiles, the flux -- is fetched by
// one thread with cp.async.bulk.tensor (TMA) into a ring of STAGES
// shared-memory buffers, STAGES-1 planes ahead of the plane being computed,
// completion tracked by one mbarrier per stage.  Compute threads read only
// shared memory and registers; results are stored straight to global.
//
// TMA boxes (innermost first; the fourth dimension spans the 3 components):
//   E kernel: I halo box {36, TY+1, 1, 3} at (z0-4, y0-1, x)  (z-1, y-1 halo)
//             V own box  {32, TY, 1, 3}   at (z0, y0, x)
//             E index    {32, TY, 1}      at (z0, y0, x)
//             V-flux box {32, TY, 1, 3}   (UPML tiles only)
//             Lorentz/Drude state boxes {32, TY, 1, 3} (tile planes that
//             hold such nodes, from a per-tile-plane flag array)
//   H kernel: V halo box {36, TY+1, 1, 3} at (z0, y0, x)      (z+1, y+1 halo)
//             I own box  {32, TY, 1, 3}, H index box, I-flux box
// The innermost start coordinate is always a multiple of 4 floats (16 B);
// out-of-range parts of a box (z<0, y<0, beyond the grid) read zeros.
//
// Every wait on an mbarrier is bounded by a clock budget; on expiry the block
// sets value 4 (bit 2) of the engine's error word, stops computing (the whole block
// leaves the plane loop together via __syncthreads_or), waits -- again with
// a budget -- for the copies it has in flight, and returns.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include "kernels.cuh"
#include "node.cuh"

namespace wipems {

constexpr int TMA_MAX_STAGES = 8;
// tile rows (y) per block.  Single jobs: 32 (z) x 4 tiles of 128 threads,
// measured faster than 32 x 8 (L256 272.6 vs 277.8 us per step, D192 210.8
// vs 218) and than 32 x 2 (321 us: the y halo row costs half a tile).
// Batches: 32 x 8 -- a persistent block pays a ring prologue per work item,
// and with half-size items the B96 batch fell from 44.7 to 33.8 G.
constexpr int TMA_TY = 4;
constexpr int BATCH_TY = 8;  // default tile rows of the batched kernels (4 is the other choice)
// The batched kernels are compiled for 1024 resident threads per SM
// (__launch_bounds__(TY * 32, 1024 / (32 * TY))), which caps their registers
// at 64: the per-job descriptor fields they read from global memory cost
// registers that the single-job kernels take from constant memory.
constexpr unsigned long long TMA_WAIT_CYCLES = 4000000000ull;  // ~2 s at 2 GHz

struct TmaMaps {
    CUtensorMap I_halo, I_own, V_halo, V_own, FV_own, FI_own, idxE, idxH, AV_own, LV_own;
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

// Tensor maps that live in global memory (the batched kernels' per-job maps,
// written by host copies) are read through the tensormap proxy: an acquire
// fence on each 128-byte map orders those writes before the TMA reads them.
__device__ __forceinline__ void tensormap_acquire(const TmaMaps* m) {
    const char* p = reinterpret_cast<const char*>(m);
#pragma unroll
    for (int k = 0; k < (int)(sizeof(TmaMaps) / 128); ++k)
        asm volatile("fence.proxy.tensormap::generic.acquire.sys [%0], 128;" ::"l"(p + 128 * k) : "memory");
}

// stage layout (floats, every buffer 128-byte aligned); ADE adds the two
// Lorentz/Drude state boxes (voltage kernel only)
template <typename IdxT, bool UPML, bool ADE = false, int TY = TMA_TY>
struct StageLayout {
    static constexpr int HW = 36;                               // halo box row width
    static constexpr int HALO = 3 * (TY + 1) * HW;          // halo box, 3 components
    static constexpr int HALO_A = (HALO + 31) / 32 * 32;
    static constexpr int OWN = 3 * TY * 32;                  // own box, 3 components
    static constexpr int IDX = TY * 32 * (int)sizeof(IdxT) / 4;
    static constexpr int IDX_A = (IDX + 31) / 32 * 32;
    static constexpr int FLUX = UPML ? OWN : 0;
    static constexpr int OFF_FLUX = HALO_A + OWN + IDX_A;
    static constexpr int OFF_ADE = OFF_FLUX + FLUX;              // ADE state, then Lorentz state
    static constexpr int STAGE = OFF_ADE + (ADE ? 2 * OWN : 0);  // floats
    static constexpr int HALO_BYTES = HALO * 4;
    static constexpr int OWN_BYTES = OWN * 4;
    static constexpr int IDX_BYTES = TY * 32 * (int)sizeof(IdxT);
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

// A plane's place in the mbarrier ring: plane q of a block's running count
// sits in stage q % STAGES and completes phase (q / STAGES) & 1 of that
// stage's barrier.  The position is derived once per tile and then stepped
// plane by plane, so the loops carry no integer division by the runtime
// stage count.
struct RingPos {
    int s;
    uint32_t ph;
    __device__ __forceinline__ RingPos(uint32_t q, int stages)
        : s((int)(q % (uint32_t)stages)), ph((q / (uint32_t)stages) & 1u) {}
    __device__ __forceinline__ void next(int stages) {
        if (++s == stages) {
            s = 0;
            ph ^= 1u;
        }
    }
};

// ------------------------------------------------------------- E half-step
// One tile of the voltage update: the 32 x TY tile (bx, by) over the
// x-chunk bz.  ring counts the planes this block has pushed through its
// mbarrier ring so far (the ring persists across the tiles of a persistent
// block).  Returns false if a bounded wait gave up.
// per (x, y-tile, z-tile) Lorentz/Drude flags of the voltage kernel's tiles:
// bit 0 = an ADE node, bit 1 = a Lorentz node in that tile plane
// (the array has TMA_TY-row granularity; a TY-row tile ORs the rows it spans)
template <int TY>
__device__ __forceinline__ uint32_t ade_tile_flags(const DevGrid& g, int x, int bx, int by) {
    if (!g.ade_tile) return 0u;
    const int ZT = (g.Nz + 31) / 32, YT = (g.Ny + TMA_TY - 1) / TMA_TY;
    uint32_t f = 0u;
#pragma unroll
    for (int k = 0; k < TY / TMA_TY; ++k) {
        const int r = by * (TY / TMA_TY) + k;
        if (r < YT) f |= (uint32_t)__ldg(g.ade_tile + ((long long)x * YT + r) * ZT + bx);
    }
    return f;
}

template <typename IdxT, int FEAT, bool GEO, int TY = TMA_TY>
__device__ __forceinline__ bool volt_tile(const DevGrid& g, const TmaMaps& m, const TileInfo& ti, int bx, int by,
                                          int bz, int XC, int STAGES, float* smem, uint64_t* bars, uint32_t& ring,
                                          int numTS) {
    constexpr bool UPML = (FEAT & FEAT_UPML) != 0;
    constexpr bool ADE = (FEAT & FEAT_ADE) != 0;
    using L = StageLayout<IdxT, UPML, ADE, TY>;
    constexpr int HW = L::HW;
    const int tz = threadIdx.x, ty = threadIdx.y;
    const int tid = ty * 32 + tz;
    const int z0 = bx * 32, y0 = by * TY;
    const int z = z0 + tz, y = y0 + ty;
    const int x0 = bz * XC;
    const int x1 = min(x0 + XC, ti.ne[0]);
    const int nplanes = x1 - x0;
    const bool valid = (y < ti.ne[1]) && (z < ti.ne[2]);
    const long long C = g.comp;
    const int zl = min(z0 + 31, g.Nz - 1), yl = min(y0 + TY - 1, g.Ny - 1);
    const uint32_t base = ring;

    auto issue = [&](int r, int s) {  // thread 0: plane x0+r into ring stage s
        const int x = x0 + r;
        float* st = smem + (size_t)s * L::STAGE;
        const bool up = UPML && tile_has_upml(ti, x, y0, yl, z0, zl);
        const uint32_t af = ADE ? ade_tile_flags<TY>(g, x, bx, by) : 0u;
        const uint32_t bytes = L::HALO_BYTES + L::OWN_BYTES + L::IDX_BYTES + (up ? L::OWN_BYTES : 0) +
                               ((af & 1u) ? L::OWN_BYTES : 0) + ((af & 2u) ? L::OWN_BYTES : 0);
        mbar_expect_tx(&bars[s], bytes);
        tma_4d(st, &m.I_halo, &bars[s], z0 - 4, y0 - 1, x, 0);
        tma_4d(st + L::HALO_A, &m.V_own, &bars[s], z0, y0, x, 0);
        tma_3d(st + L::HALO_A + L::OWN, &m.idxE, &bars[s], z0, y0, x);
        if (up) tma_4d(st + L::OFF_FLUX, &m.FV_own, &bars[s], z0, y0, x, 0);
        if (af & 1u) tma_4d(st + L::OFF_ADE, &m.AV_own, &bars[s], z0, y0, x, 0);
        if (af & 2u) tma_4d(st + L::OFF_ADE + L::OWN, &m.LV_own, &bars[s], z0, y0, x, 0);
    };

    int issued = 0;
    if (tid == 0) {
        fence_proxy_async();
        for (RingPos ip(base, STAGES); issued < min(STAGES - 1, nplanes); ++issued, ip.next(STAGES))
            issue(issued, ip.s);
    }
    float p1 = 0.f, p2 = 0.f;  // I1, I2 at x-1
    const long long yz = (long long)y * g.Nzp + z;
    if (valid && x0 > 0) {
        const long long o = (long long)(x0 - 1) * g.sx + yz;
        p1 = g.I[C + o];
        p2 = g.I[2 * C + o];
    }
    // geometry factors: y / z parts are fixed per thread, x part per plane
    float gyE = 0.f, gyI = 0.f, gzE = 0.f, gzI = 0.f;
    if (GEO && valid) {
        const int S = g.geo_stride;
        gyE = __ldg(g.geo + g.Nx + y);
        gyI = __ldg(g.geo + S + g.Nx + y);
        gzE = __ldg(g.geo + g.Nx + g.Ny + z);
        gzI = __ldg(g.geo + S + g.Nx + g.Ny + z);
    }
    float* Vp = g.V + (long long)x0 * g.sx + yz;  // node (x0, y, z), advanced by sx per plane
    bool aborted = false;
    int r = 0;
    RingPos cp(base, STAGES);  // stage of plane r
    for (; r < nplanes; ++r, Vp += g.sx, cp.next(STAGES)) {
        if (tid == 0 && issued < nplanes && issued == r + STAGES - 1) {
            // plane r + STAGES - 1 goes into the stage plane r - 1 freed
            fence_proxy_async();
            issue(issued, cp.s == 0 ? STAGES - 1 : cp.s - 1);
            ++issued;
        }
        const bool ok = mbar_wait(&bars[cp.s], cp.ph);
        const int x = x0 + r;
        const float* st = smem + (size_t)cp.s * L::STAGE;
        float c1 = 0.f, c2 = 0.f;
        if (ok && valid) {
            const int hi = (ty + 1) * HW + 4 + tz;  // own position in the halo box
            const float* sI0 = st;
            const float* sI1 = st + (TY + 1) * HW;
            const float* sI2 = st + 2 * (TY + 1) * HW;
            const float c0 = sI0[hi];
            c1 = sI1[hi];
            c2 = sI2[hi];
            const float i2ym = (y > 0) ? sI2[hi - HW] : c2;
            const float i0ym = (y > 0) ? sI0[hi - HW] : c0;
            const float i1zm = (z > 0) ? sI1[hi - 1] : c1;
            const float i0zm = (z > 0) ? sI0[hi - 1] : c0;
            const float i2xm = (x > 0) ? p2 : c2;
            const float i1xm = (x > 0) ? p1 : c1;
            float curl[3];
            curl[0] = __fadd_rn(__fsub_rn(__fsub_rn(c2, i2ym), c1), i1zm);
            curl[1] = __fadd_rn(__fsub_rn(__fsub_rn(c0, i0zm), c2), i2xm);
            curl[2] = __fadd_rn(__fsub_rn(__fsub_rn(c1, i1xm), c0), i0ym);
            const int oi = ty * 32 + tz;
            const float* sV = st + L::HALO_A;
            const uint32_t t = (uint32_t)reinterpret_cast<const IdxT*>(st + L::HALO_A + L::OWN)[oi];
            const bool up = UPML && tile_has_upml(ti, x, y0, yl, z0, zl);
            const float* sF = up ? st + L::OFF_FLUX + oi : nullptr;
            const uint32_t af = ADE ? ade_tile_flags<TY>(g, x, bx, by) : 0u;
            const float* sA = (af & 1u) ? st + L::OFF_ADE + oi : nullptr;
            const float* sL = (af & 2u) ? st + L::OFF_ADE + L::OWN + oi : nullptr;
            float v[3] = {sV[oi], sV[TY * 32 + oi], sV[2 * TY * 32 + oi]};
            GeoF gf;
            if (GEO) {
                const float gxE = __ldg(g.geo + x), gxI = __ldg(g.geo + g.geo_stride + x);
                gf.f[0][0] = gxE; gf.f[0][1] = gyI; gf.f[0][2] = gzI;
                gf.f[1][0] = gyE; gf.f[1][1] = gzI; gf.f[1][2] = gxI;
                gf.f[2][0] = gzE; gf.f[2][1] = gxI; gf.f[2][2] = gyI;
            }
            update_node<false, FEAT, GEO>(g, v, curl, t, (long long)x * g.sx + yz, numTS, sF, TY * 32, gf,
                                          nullptr, true, sA, sL);
            Vp[0] = v[0];
            Vp[C] = v[1];
            Vp[2 * C] = v[2];
        }
        p1 = c1;
        p2 = c2;
        if (__syncthreads_or(!ok)) {
            aborted = true;
            break;
        }
    }
    ring = base + (uint32_t)nplanes;
    if (aborted && tid == 0) {
        atomicOr(ti.d_err, 4);
        // wait (bounded) for the copies this block still has in flight
        for (int k = r; k < issued; ++k) {
            const uint32_t q = base + (uint32_t)k;
            mbar_wait(&bars[q % (uint32_t)STAGES], (q / (uint32_t)STAGES) & 1u);
        }
    }
    return !aborted;
}

// ------------------------------------------------------------- H half-step
// One tile of the current update (see volt_tile).  es/ec/hs/hc: the
// thread's Kahan sums of V^2 and I^2, accumulated when energy is set.
template <typename IdxT, int FEAT, bool GEO, int TY = TMA_TY>
__device__ __forceinline__ bool curr_tile(const DevGrid& g, const TmaMaps& m, const TileInfo& ti, int bx, int by,
                                          int bz, int XC, int STAGES, float* smem, uint64_t* bars, uint32_t& ring,
                                          int numTS, bool energy) {
    constexpr bool UPML = (FEAT & FEAT_UPML) != 0;
    using L = StageLayout<IdxT, UPML, false, TY>;
    constexpr int HW = L::HW;
    const int tz = threadIdx.x, ty = threadIdx.y;
    const int tid = ty * 32 + tz;
    const int z0 = bx * 32, y0 = by * TY;
    const int z = z0 + tz, y = y0 + ty;
    const int x0 = bz * XC;
    const int x1 = min(x0 + XC, g.Nx - 1);
    const int nplanes = x1 - x0;      // planes updated
    const int nload = nplanes + 1;    // plane x1 is read as the x+1 neighbour
    const bool active = (z < g.Nz - 1) && (y < g.Ny - 1);
    const long long C = g.comp;
    const int zl = min(z0 + 31, g.Nz - 1), yl = min(y0 + TY - 1, g.Ny - 1);
    const uint32_t base = ring;

    auto issue = [&](int r, int s) {  // thread 0: plane x0+r into ring stage s
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
            tma_3d(st + L::HALO_A + L::OWN, &m.idxH, &bars[s], z0, y0, x);
        }
        if (up) tma_4d(st + L::OFF_FLUX, &m.FI_own, &bars[s], z0, y0, x, 0);
    };

    int issued = 0;
    if (nplanes > 0 && tid == 0) {
        fence_proxy_async();
        for (RingPos ip(base, STAGES); issued < min(STAGES - 1, nload); ++issued, ip.next(STAGES))
            issue(issued, ip.s);
    }
    const long long yz = (long long)y * g.Nzp + z;
    float gyE = 0.f, gyI = 0.f, gzE = 0.f, gzI = 0.f;  // dH / iM parts
    if (GEO && active) {
        const int S = g.geo_stride;
        gyE = __ldg(g.geo + 2 * S + g.Nx + y);
        gyI = __ldg(g.geo + 3 * S + g.Nx + y);
        gzE = __ldg(g.geo + 2 * S + g.Nx + g.Ny + z);
        gzI = __ldg(g.geo + 3 * S + g.Nx + g.Ny + z);
    }
    float* Ip = g.I + (long long)x0 * g.sx + yz;
    bool aborted = false;
    int r = 0;
    RingPos cp(base, STAGES);  // stage of plane r
    for (; r < nplanes; ++r, Ip += g.sx, cp.next(STAGES)) {
        if (tid == 0 && issued < nload && issued == r + STAGES - 1) {
            // plane r + STAGES - 1 goes into the stage plane r - 1 freed
            fence_proxy_async();
            issue(issued, cp.s == 0 ? STAGES - 1 : cp.s - 1);
            ++issued;
        }
        const int s = cp.s;
        const int sn = s + 1 == STAGES ? 0 : s + 1;  // plane r + 1 (its V is the x+1 neighbour)
        bool ok = mbar_wait(&bars[s], cp.ph);
        ok = ok && mbar_wait(&bars[sn], cp.ph ^ (uint32_t)(sn == 0));
        const int x = x0 + r;
        float ev[3] = {0.f, 0.f, 0.f}, eh[3] = {0.f, 0.f, 0.f};  // energy terms of this node
        if (ok && active) {
            const float* st = smem + (size_t)s * L::STAGE;
            const float* stn = smem + (size_t)sn * L::STAGE;
            const float* sV0 = st;
            const float* sV1 = st + (TY + 1) * HW;
            const float* sV2 = st + 2 * (TY + 1) * HW;
            const int hi = ty * HW + tz;
            const float c0 = sV0[hi], c1 = sV1[hi], c2 = sV2[hi];
            const float n1 = stn[(TY + 1) * HW + hi];
            const float n2 = stn[2 * (TY + 1) * HW + hi];
            float curl[3];
            curl[0] = __fadd_rn(__fsub_rn(__fsub_rn(c2, sV2[hi + HW]), c1), sV1[hi + 1]);
            curl[1] = __fadd_rn(__fsub_rn(__fsub_rn(c0, sV0[hi + 1]), c2), n2);
            curl[2] = __fadd_rn(__fsub_rn(__fsub_rn(c1, n1), c0), sV0[hi + HW]);
            const int oi = ty * 32 + tz;
            const float* sI = st + L::HALO_A;
            const uint32_t t = (uint32_t)reinterpret_cast<const IdxT*>(st + L::HALO_A + L::OWN)[oi];
            const bool up = UPML && tile_has_upml(ti, x, y0, yl, z0, zl);
            const float* sF = up ? st + L::OFF_FLUX + oi : nullptr;
            float cu[3] = {sI[oi], sI[TY * 32 + oi], sI[2 * TY * 32 + oi]};
            GeoF gf;
            if (GEO) {
                const int S = g.geo_stride;
                const float gxE = __ldg(g.geo + 2 * S + x), gxI = __ldg(g.geo + 3 * S + x);
                gf.f[0][0] = gxE; gf.f[0][1] = gyI; gf.f[0][2] = gzI;
                gf.f[1][0] = gyE; gf.f[1][1] = gzI; gf.f[1][2] = gxI;
                gf.f[2][0] = gzE; gf.f[2][1] = gxI; gf.f[2][2] = gyI;
            }
            update_node<true, FEAT, GEO>(g, cu, curl, t, (long long)x * g.sx + yz, numTS, sF, TY * 32, gf);
            Ip[0] = cu[0];
            Ip[C] = cu[1];
            Ip[2 * C] = cu[2];
            ev[0] = c0; ev[1] = c1; ev[2] = c2;
            eh[0] = cu[0]; eh[1] = cu[1]; eh[2] = cu[2];
        }
        if (energy)  // Engine_Interface_FDTD::CalcFastEnergy terms of segment (x, y, bx)
            energy_segment(g, x, y, bx, ok && active, ok && y < g.Ny - 1 && z0 < g.Nz - 1, ev[0], ev[1], ev[2],
                           eh[0], eh[1], eh[2]);
        if (__syncthreads_or(!ok)) {
            aborted = true;
            break;
        }
    }
    ring = base + (uint32_t)(nplanes > 0 ? nload : 0);
    if (aborted && tid == 0) {
        atomicOr(ti.d_err, 4);
        for (int k = r; k < issued; ++k) {
            const uint32_t q = base + (uint32_t)k;
            mbar_wait(&bars[q % (uint32_t)STAGES], (q / (uint32_t)STAGES) & 1u);
        }
    }
    return !aborted;
}

__device__ __forceinline__ float* aligned_smem(float* raw) {
    return reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(raw) + 127) & ~(uintptr_t)127);
}

__device__ __forceinline__ void init_ring(uint64_t* bars, int STAGES) {
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        for (int s = 0; s < STAGES; ++s) mbar_init(&bars[s], 1);
        fence_barrier_init();
    }
    __syncthreads();
}

// ---------------------------------------------------------- single job
// TY: tile rows (4 or 8; the tensor maps' box height matches)
template <typename IdxT, int FEAT, bool GEO, int TY>
__global__ void __launch_bounds__(TY * 32) k_volt_tma(const DevGrid g, const __grid_constant__ TmaMaps m,
                                                      const TileInfo ti, int ts_off, int XC, int STAGES) {
    using L = StageLayout<IdxT, (FEAT & FEAT_UPML) != 0, (FEAT & FEAT_ADE) != 0, TY>;
    extern __shared__ __align__(128) float smem_raw[];
    float* smem = aligned_smem(smem_raw);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + (size_t)L::STAGE * STAGES);
    if (*g.d_done) return;
    init_ring(bars, STAGES);
    uint32_t ring = 0;
    volt_tile<IdxT, FEAT, GEO, TY>(g, m, ti, blockIdx.x, blockIdx.y, blockIdx.z, XC, STAGES, smem, bars, ring,
                                   *g.d_ts + ts_off);
}

template <typename IdxT, int FEAT, bool GEO, bool ENERGY, int TY>
__global__ void __launch_bounds__(TY * 32) k_curr_tma(const DevGrid g, const __grid_constant__ TmaMaps m,
                                                      const TileInfo ti, int ts_off, int XC, int STAGES) {
    using L = StageLayout<IdxT, (FEAT & FEAT_UPML) != 0, false, TY>;
    extern __shared__ __align__(128) float smem_raw[];
    float* smem = aligned_smem(smem_raw);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + (size_t)L::STAGE * STAGES);
    if (*g.d_done) return;
    init_ring(bars, STAGES);
    uint32_t ring = 0;
    // x-chunks in descending order: blocks are dispatched roughly in
    // blockIdx order, and the voltage kernel before this one ended on the
    // highest chunks, whose voltages (just written) and currents (just read)
    // are still partly in L2.  The next voltage kernel, in ascending order,
    // starts where this one ends.  No block reads what another block of the
    // same kernel writes, so the order does not change any result.
    curr_tile<IdxT, FEAT, GEO, TY>(g, m, ti, blockIdx.x, blockIdx.y, gridDim.z - 1 - blockIdx.z, XC, STAGES, smem,
                                   bars, ring, *g.d_ts + ts_off, ENERGY);
}

// ---------------------------------------------------------- batched jobs
// One job of a batch: its grid, UPML geometry, tensor maps (in global
// memory) and probe interval (0 = no sampling).
struct BatchJob {
    DevGrid g;
    TileInfo ti;
    const TmaMaps* maps;
    int interval;
    int energy;  // the job records energies on its sample steps
    int pad[2];
};

// Work item of a persistent batched kernel: job, tile (bx, by), x-chunk bz.
struct WorkItem {
    int job, bx, by, bz;
};

// Persistent voltage half-step over the work items of many jobs: block b
// takes items b, b + gridDim.x, ...  Every job's numTS is read from its own
// counter, so jobs need not be in step.
template <typename IdxT, int FEAT, bool GEO, int TY = BATCH_TY>
__global__ void __launch_bounds__(TY * 32, 1024 / (32 * TY)) k_volt_batch(const BatchJob* __restrict__ jobs,
                                                            const WorkItem* __restrict__ items, int nitems, int XC,
                                                            int STAGES) {
    using L = StageLayout<IdxT, (FEAT & FEAT_UPML) != 0, (FEAT & FEAT_ADE) != 0, TY>;
    extern __shared__ __align__(128) float smem_raw[];
    float* smem = aligned_smem(smem_raw);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + (size_t)L::STAGE * STAGES);
    init_ring(bars, STAGES);
    uint32_t ring = 0;
    int last_job = -1;
    for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
        const WorkItem w = items[it];
        const BatchJob& J = jobs[w.job];
        if (*J.g.d_done) continue;  // the job met its end criterion
        if (w.job != last_job) {
            if (threadIdx.x == 0 && threadIdx.y == 0) tensormap_acquire(J.maps);
            last_job = w.job;
        }
        if (!volt_tile<IdxT, FEAT, GEO, TY>(J.g, *J.maps, J.ti, w.bx, w.by, w.bz, XC, STAGES, smem, bars, ring,
                                        *J.g.d_ts))
            break;
    }
}

template <typename IdxT, int FEAT, bool GEO, int TY = BATCH_TY>
__global__ void __launch_bounds__(TY * 32, 1024 / (32 * TY)) k_curr_batch(const BatchJob* __restrict__ jobs,
                                                            const WorkItem* __restrict__ items, int nitems, int XC,
                                                            int STAGES) {
    using L = StageLayout<IdxT, (FEAT & FEAT_UPML) != 0, false, TY>;
    extern __shared__ __align__(128) float smem_raw[];
    float* smem = aligned_smem(smem_raw);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + (size_t)L::STAGE * STAGES);
    init_ring(bars, STAGES);
    uint32_t ring = 0;
    int last_job = -1;
    for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
        const WorkItem w = items[it];
        const BatchJob& J = jobs[w.job];
        if (*J.g.d_done) continue;
        if (w.job != last_job) {
            if (threadIdx.x == 0 && threadIdx.y == 0) tensormap_acquire(J.maps);
            last_job = w.job;
        }
        // energy on the job's sample steps (the sample after this step)
        const int numTS = *J.g.d_ts;
        const bool energy = J.interval > 0 && J.energy && ((numTS + 1) % J.interval) == 0;
        const bool ok = curr_tile<IdxT, FEAT, GEO, TY>(J.g, *J.maps, J.ti, w.bx, w.by, w.bz, XC, STAGES, smem, bars,
                                                   ring, numTS, energy);
        if (!ok) break;
    }
}

}  // namespace wipems
