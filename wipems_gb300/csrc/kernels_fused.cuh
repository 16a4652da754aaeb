// Fused single-pass timestep kernel: the voltage and the current half-step of
// one timestep in one march over x, for grids without Lorentz/Drude nodes and
// without factorized geometry.
//
// The two-pass kernels read V and I twice per timestep and write each once
// (76 B per node with 16-bit indices); this one reads each once and writes
// each once (52 B per node).  It keeps the same per-node arithmetic as the
// two-pass kernels (node.cuh), so results are bit-identical.
//
// Dependencies.  H at node (x, y, z) needs the NEW V at x, x+1, y+1 and z+1;
// E at (x, y, z) needs the OLD I at x-1, y-1, z-1.  A block owns a tile of
// 32 (z) x 8 (y) H nodes over an x-chunk and marches over x with E one plane
// ahead of H; its ten warps update the 32 x 8 E nodes of the tile, the row
// above it and the column beside it in one pass, then eight of them the H
// nodes.  The new V it needs just outside its tile (row y0+8, column
// z0+32, plane x1) belongs to neighbouring blocks, which may not have
// computed it yet -- so the block recomputes those E nodes itself (about 16 %
// extra E work), and fields are double-buffered so that nobody overwrites an
// old value a neighbour still needs: the step at numTS reads buffer numTS&1
// and writes buffer (numTS+1)&1.  The UPML voltage flux is double-buffered
// the same way (redundant E nodes read it); the current flux is updated in
// place (H has no redundancy).  Only the owning block stores a node.
//
// Per x-plane the ring stage holds (TMA, 16-byte-aligned z starts):
//   I halo  box {40, 10, 1, 3} at (z0-4, y0-1, x)  old I, y-1 / z-1 halo
//   V ext   box {36,  9, 1, 3} at (z0,   y0,   x)  old V of the E region
//   E index box {40,  9, 1}    at (z0,   y0,   x)
//   H index box {32,  8, 1}    at (z0,   y0,   x)
//   V flux  box {36,  9, 1, 3}, I flux box {32, 8, 1, 3}  (UPML tiles)
// and the new V of planes x and x+1 stays in shared memory for H.  Waits are
// bounded as in kernels_tma.cuh (error bit 4, the block leaves together).
#pragma once

#include "kernels_tma.cuh"

namespace wipems {

constexpr int FU_TY = 8;          // H tile rows
constexpr int FU_WARPS = FU_TY + 2;  // + one warp for E row y0+8, one for E column z0+32
constexpr int FU_EH = FU_TY + 1;  // E rows: the tile and the row above it
constexpr int FU_IW = 40;         // I halo row width  (z0-4 .. z0+35)
constexpr int FU_IH = FU_TY + 2;  // I halo rows       (y0-1 .. y0+8)
constexpr int FU_VW = 36;         // V / V-flux / new-V row width (z0 .. z0+35)
constexpr int FU_XW = 40;         // E index row width (z0 .. z0+39)

__host__ __device__ constexpr int fu_a32(int n) { return (n + 31) / 32 * 32; }

struct FusedMaps {
    CUtensorMap I_halo[2];  // per field buffer
    CUtensorMap V_ext[2];
    CUtensorMap FV_ext[2];
    CUtensorMap FI_own;
    CUtensorMap idxE_ext;
    CUtensorMap idxH_own;
};

// shared-memory layout in floats; every box starts 128-byte aligned
template <typename IdxE, typename IdxH, bool UPML>
struct FusedLayout {
    static constexpr int IC = FU_IH * FU_IW;  // I halo, one component
    static constexpr int VC = FU_EH * FU_VW;  // V ext / new V, one component
    static constexpr int IH = fu_a32(3 * IC);
    static constexpr int VX = fu_a32(3 * VC);
    static constexpr int XE = fu_a32(FU_EH * FU_XW * (int)sizeof(IdxE) / 4);
    static constexpr int XH = fu_a32(FU_TY * 32 * (int)sizeof(IdxH) / 4);
    static constexpr int FX = UPML ? VX : 0;
    static constexpr int FH = UPML ? 3 * FU_TY * 32 : 0;
    static constexpr int O_VX = IH, O_XE = O_VX + VX, O_XH = O_XE + XE, O_FX = O_XH + XH, O_FH = O_FX + FX;
    static constexpr int STAGE = O_FH + FH;
    static constexpr uint32_t IH_B = 3 * IC * 4;
    static constexpr uint32_t VX_B = 3 * VC * 4;
    static constexpr uint32_t XE_B = FU_EH * FU_XW * sizeof(IdxE);
    static constexpr uint32_t XH_B = FU_TY * 32 * sizeof(IdxH);
    static constexpr uint32_t FH_B = 3 * FU_TY * 32 * 4;
    static constexpr int VN = fu_a32(3 * VC);  // one plane of new V
    static size_t smem(int stages) {
        return ((size_t)STAGE * stages + 2 * (size_t)VN) * 4 + 8 * TMA_MAX_STAGES + 128;
    }
};

template <typename IdxE, typename IdxH, int FEAT, bool ENERGY>
__global__ void __launch_bounds__(FU_WARPS * 32) k_step_fused(const DevGrid g, const __grid_constant__ FusedMaps m,
                                                           const TileInfo ti, int ts_off, int XC, int STAGES) {
    constexpr bool UPML = (FEAT & FEAT_UPML) != 0;
    using L = FusedLayout<IdxE, IdxH, UPML>;
    extern __shared__ __align__(128) float smem_raw[];
    float* smem = aligned_smem(smem_raw);
    float* vnew_s = smem + (size_t)L::STAGE * STAGES;  // [2][VN]: new V of two planes
    uint64_t* bars = reinterpret_cast<uint64_t*>(vnew_s + 2 * L::VN);
    if (*g.d_done) return;
    init_ring(bars, STAGES);

    const int tz = threadIdx.x, ty = threadIdx.y;
    const int tid = ty * 32 + tz;
    const int z0 = blockIdx.x * 32, y0 = blockIdx.y * FU_TY;
    const int x0 = blockIdx.z * XC;
    const int x1 = min(x0 + XC, g.Nx - 1);  // H planes [x0, x1)
    const int nplanes = x1 - x0;
    const int nload = nplanes + 2;          // ring planes x0-1 .. x1
    const int numTS = *g.d_ts + ts_off;
    const int p = numTS & 1;                // buffer holding the fields at numTS
    float* Vn = p ? g.V : g.V2;             // buffer written: (numTS + 1) & 1
    float* In = p ? g.I : g.I2;
    float* FVn = p ? g.FV : g.FV2;
    const long long C = g.comp;
    const int yl = min(y0 + FU_TY - 1, g.Ny - 1), zl = min(z0 + 31, g.Nz - 1);
    const int yle = min(y0 + FU_TY, g.Ny - 1), zle = min(z0 + 32, g.Nz - 1);
    const bool own_row8 = (y0 + FU_TY == g.Ny - 1);  // no tile starts at the last line
    const bool own_col32 = (z0 + 32 == g.Nz - 1);

    auto issue = [&](int q) {  // thread 0: ring plane q (x = x0 - 1 + q)
        const int s = q % STAGES;
        const int x = x0 - 1 + q;
        float* st = smem + (size_t)s * L::STAGE;
        const bool needE = q >= 1;
        const bool needH = q >= 1 && q <= nplanes;
        const bool upE = UPML && needE && tile_has_upml(ti, x, y0, yle, z0, zle);
        const bool upH = UPML && needH && tile_has_upml(ti, x, y0, yl, z0, zl);
        const uint32_t bytes = L::IH_B + (needE ? L::VX_B + L::XE_B : 0u) + (upE ? L::VX_B : 0u) +
                               (needH ? L::XH_B : 0u) + (upH ? L::FH_B : 0u);
        mbar_expect_tx(&bars[s], bytes);
        tma_4d(st, &m.I_halo[p], &bars[s], z0 - 4, y0 - 1, x, 0);
        if (needE) {
            tma_4d(st + L::O_VX, &m.V_ext[p], &bars[s], z0, y0, x, 0);
            tma_3d(st + L::O_XE, &m.idxE_ext, &bars[s], z0, y0, x);
            if (upE) tma_4d(st + L::O_FX, &m.FV_ext[p], &bars[s], z0, y0, x, 0);
        }
        if (needH) {
            tma_3d(st + L::O_XH, &m.idxH_own, &bars[s], z0, y0, x);
            if (upH) tma_4d(st + L::O_FH, &m.FI_own, &bars[s], z0, y0, x, 0);
        }
    };
    auto stage = [&](int q) { return smem + (size_t)(q % STAGES) * L::STAGE; };
    auto wait = [&](int q) { return mbar_wait(&bars[q % STAGES], (uint32_t)(q / STAGES) & 1u); };

    // E update of node (ey, ez) of the E region at plane x; sc / sp: ring
    // stages of planes x and x-1; the new V goes to vn (shared) and, for the
    // owner, to the new buffer.
    const GeoF gf{};
    auto e_node = [&](int ey, int ez, int x, const float* sc, const float* sp, float* vn, bool upE) {
        const int y = y0 + ey, z = z0 + ez;
        const int vi = ey * FU_VW + ez;
        const float* sV = sc + L::O_VX;
        float v[3] = {sV[vi], sV[L::VC + vi], sV[2 * L::VC + vi]};
        if (x >= 0 && x < ti.ne[0] && y < ti.ne[1] && z < ti.ne[2]) {
            const int hi = (ey + 1) * FU_IW + ez + 4;
            const float c0 = sc[hi], c1 = sc[L::IC + hi], c2 = sc[2 * L::IC + hi];
            const float i2ym = (y > 0) ? sc[2 * L::IC + hi - FU_IW] : c2;
            const float i0ym = (y > 0) ? sc[hi - FU_IW] : c0;
            const float i1zm = (z > 0) ? sc[L::IC + hi - 1] : c1;
            const float i0zm = (z > 0) ? sc[hi - 1] : c0;
            const float i1xm = (x > 0) ? sp[L::IC + hi] : c1;
            const float i2xm = (x > 0) ? sp[2 * L::IC + hi] : c2;
            float curl[3];
            curl[0] = __fadd_rn(__fsub_rn(__fsub_rn(c2, i2ym), c1), i1zm);
            curl[1] = __fadd_rn(__fsub_rn(__fsub_rn(c0, i0zm), c2), i2xm);
            curl[2] = __fadd_rn(__fsub_rn(__fsub_rn(c1, i1xm), c0), i0ym);
            const uint32_t t = (uint32_t)reinterpret_cast<const IdxE*>(sc + L::O_XE)[ey * FU_XW + ez];
            const float* sF = upE ? sc + L::O_FX + vi : nullptr;
            const bool own = (ey < FU_TY || own_row8) && (ez < 32 || own_col32) && (x < x1 || x == g.Nx - 1);
            const long long o = (long long)x * g.sx + (long long)y * g.Nzp + z;
            update_node<false, FEAT, false>(g, v, curl, t, o, numTS, sF, L::VC, gf, FVn, own);
            if (own) {
                Vn[o] = v[0];
                Vn[C + o] = v[1];
                Vn[2 * C + o] = v[2];
            }
        }
        vn[vi] = v[0];
        vn[L::VC + vi] = v[1];
        vn[2 * L::VC + vi] = v[2];
    };
    // E of a whole plane in one pass: warps 0..7 their own node, warp 8 the
    // row y0+8 (z0..z0+31), warp 9 the column z0+32 (y0..y0+8)
    auto e_plane = [&](int x, const float* sc, const float* sp, float* vn) {
        const bool upE = UPML && tile_has_upml(ti, x, y0, yle, z0, zle);
        if (ty < FU_TY + 1) e_node(ty, tz, x, sc, sp, vn, upE);
        else if (tz <= FU_TY) e_node(tz, 32, x, sc, sp, vn, upE);
    };

    int issued = 0;
    if (tid == 0) {
        fence_proxy_async();
        for (; issued < min(STAGES, nload); ++issued) issue(issued);
    }
    bool aborted = false;
    int waited = 0;  // ring planes whose copies this thread saw complete, in order
    // prologue: E at plane x0 (ring planes 0 and 1)
    {
        bool ok = wait(0);
        if (ok) waited = 1;
        ok = ok && wait(1);
        if (ok) waited = 2;
        if (ok) e_plane(x0, stage(1), stage(0), vnew_s);
        if (__syncthreads_or(!ok)) aborted = true;
        if (!aborted && tid == 0 && issued < nload) {  // ring plane 0 is free
            fence_proxy_async();
            issue(issued);
            ++issued;
        }
    }
    const int y = y0 + ty, z = z0 + tz;
    const bool hact = (ty < FU_TY) && (y < g.Ny - 1) && (z < g.Nz - 1);
    for (int r = 0; r < nplanes && !aborted; ++r) {
        const int x = x0 + r;
        float* vc = vnew_s + (size_t)(r & 1) * L::VN;        // new V, plane x
        float* vx = vnew_s + (size_t)((r + 1) & 1) * L::VN;  // new V, plane x+1
        // E at plane x+1 (ring planes r+1 = x and r+2 = x+1)
        const bool ok = wait(r + 2);
        if (ok) waited = r + 3;
        if (ok) e_plane(x + 1, stage(r + 2), stage(r + 1), vx);
        if (__syncthreads_or(!ok)) {
            aborted = true;
            break;
        }
        // H at plane x (ring plane r+1)
        float ev[3] = {0.f, 0.f, 0.f}, eh[3] = {0.f, 0.f, 0.f};  // energy terms of this node
        if (hact) {
            const float* st = stage(r + 1);
            const int vi = ty * FU_VW + tz;
            const float c0 = vc[vi], c1 = vc[L::VC + vi], c2 = vc[2 * L::VC + vi];
            const float n1 = vx[L::VC + vi], n2 = vx[2 * L::VC + vi];
            float curl[3];
            curl[0] = __fadd_rn(__fsub_rn(__fsub_rn(c2, vc[2 * L::VC + vi + FU_VW]), c1), vc[L::VC + vi + 1]);
            curl[1] = __fadd_rn(__fsub_rn(__fsub_rn(c0, vc[vi + 1]), c2), n2);
            curl[2] = __fadd_rn(__fsub_rn(__fsub_rn(c1, n1), c0), vc[vi + FU_VW]);
            const int hi = (ty + 1) * FU_IW + tz + 4;
            float cu[3] = {st[hi], st[L::IC + hi], st[2 * L::IC + hi]};
            const uint32_t t = (uint32_t)reinterpret_cast<const IdxH*>(st + L::O_XH)[tid];
            const bool upH = UPML && tile_has_upml(ti, x, y0, yl, z0, zl);
            const float* sF = upH ? st + L::O_FH + tid : nullptr;
            const long long o = (long long)x * g.sx + (long long)y * g.Nzp + z;
            update_node<true, FEAT, false>(g, cu, curl, t, o, numTS, sF, FU_TY * 32, gf);
            In[o] = cu[0];
            In[C + o] = cu[1];
            In[2 * C + o] = cu[2];
            ev[0] = c0; ev[1] = c1; ev[2] = c2;
            eh[0] = cu[0]; eh[1] = cu[1]; eh[2] = cu[2];
        }
        if (ENERGY)  // segment (x, y, blockIdx.x); the halo warp (ty == FU_TY) owns none
            energy_segment(g, x, y, blockIdx.x, hact, ty < FU_TY && y < g.Ny - 1 && z0 < g.Nz - 1, ev[0], ev[1],
                           ev[2], eh[0], eh[1], eh[2]);
        __syncthreads();  // ring plane r+1 and new-V plane x are free
        if (tid == 0 && issued < nload) {
            fence_proxy_async();
            issue(issued);
            ++issued;
        }
    }
    if (aborted && tid == 0) {
        atomicOr(ti.d_err, 4);
        for (int q = waited; q < issued; ++q) wait(q);  // bounded: copies still in flight
    }
}

}  // namespace wipems
