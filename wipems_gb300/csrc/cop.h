// Compressed operator: what the device engine reads per node.
//
// The reference compresses its per-edge FP32 coefficients into unique
// tuples plus an index (Operator_SSE_Compressed::CompressOperator,
// operator_sse_compressed.cpp:120-176).  Here the same idea is applied per
// node and per half-step: every node has an E-tuple index and an H-tuple
// index (uint16 when the unique tuples fit, else uint32), and a tuple holds
// everything the fused kernel of that half-step needs for the node:
//   E: vv[3], vi[3], flags, UPML (vvp, vvfo, vvfn)[3], ADE (v_int, v_ext,
//      v_lor)[3], voltage excitation amplitude[3] and delay[3]
//   H: the same with ii/iv, the UPML current terms, the current ADE and
//      current excitation.
// Lorentz/Drude dispersion of order > 1 (several poles per material): the
// ADE terms of orders 1..3 sit in a second table (`adex`, same tuple index,
// one TAB_ADE block per extra order) with their own flag bits, and the
// kernels keep their states in [order-1][3][comp] arrays.
//
// Graded meshes: vi and iv carry the edge's geometric factor delta/A, which
// makes almost every node's tuple unique.  When the mesh is not uniform the
// tuple stores VI = vi / g(n, pos) instead, with the separable factor
//   gE(n, pos) = dE[n][p_n] * iD[nP][p_nP] * iD[nPP][p_nPP]
//   gH(n, pos) = dH[n][p_n] * iM[nP][p_nP] * iM[nPP][p_nPP]
// built from per-axis line arrays (main edge length dE, 1/dual length iD,
// dual edge length dH, 1/main length iM), and the kernels multiply it back.
// That reproduces vi within a few float ulps rather than bit-exactly.  In
// that mode the last-bit rounding variants of each coefficient kind are also
// merged onto their most frequent neighbour (at most one float step away),
// so that tuples differing only by such variants share one entry.
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

#include "../../include/wipems_fdtd.h"
#include "fdtd_host.h"

namespace wipems {

// tuple flags
constexpr uint32_t TF_UPML = 1u;
constexpr uint32_t TF_ADE = 2u;
constexpr uint32_t TF_LOR = 4u;
constexpr uint32_t TF_EXC = 8u;
// dispersion orders 1..3: ADE terms of order o at bit TF_ADEX << (o-1),
// its Lorentz pole term at bit TF_LORX << (o-1)
constexpr uint32_t TF_ADEX = 16u;
constexpr uint32_t TF_LORX = 128u;
constexpr uint32_t TF_ADEX_ALL = 7u * TF_ADEX;
constexpr int kExtraOrders = kMaxDispOrder - 1;

struct HalfTuple {
    float c[6];        // vv|ii [3], vi|iv [3] (or VI|IV in factorized mode)
    uint32_t flags;
    float u[9];        // UPML: vvp|iip [3], vvfo|iifo [3], vvfn|iifn [3]
    float a[9];        // ADE of order 0: int [3], ext [3], lor [3]
    float x[3];        // excitation amplitude
    int32_t xd[3];     // excitation delay (-1 = none)
    uint32_t pad;
    // ADE of orders 1..3 (zero unless the operator has them; tuples are
    // compared and hashed over the first kTupleBaseBytes bytes only when no
    // node has them)
    float ax[kExtraOrders][9];
    uint32_t pad2[5];
};
constexpr size_t kTupleBaseBytes = 128;
static_assert(offsetof(HalfTuple, ax) == kTupleBaseBytes, "the base tuple is 32 words");
static_assert(sizeof(HalfTuple) == 256, "the tuple with extra orders is 64 words");

// device table layout of one half (float4 units per tuple)
constexpr int TAB_MAIN = 2;  // {c0,c1,c2,c3},{c4,c5,flags,-}
constexpr int TAB_UPML = 3;  // {u0..u3},{u4..u7},{u8,-,-,-}
constexpr int TAB_ADE = 3;
constexpr int TAB_EXC = 2;   // {x0,x1,x2,-},{xd0,xd1,xd2,-}

struct HalfTables {
    uint32_t num_tuples = 0;
    bool idx16 = true;
    bool any_upml = false, any_ade = false, any_lor = false, any_exc = false;
    int adex_orders = 0;                      // extra dispersion orders present (0..3)
    bool any_lorx = false;
    std::vector<float> main, upml, ade, exc;  // float4-packed, see TAB_*
    std::vector<float> adex;                  // [order-1][tuple][TAB_ADE] float4-packed
    uint8_t* idx = nullptr;                   // [Nx][Ny][Nzp], pinned when possible
    bool pinned = false;
    size_t idx_bytes = 0;
};

}  // namespace wipems

struct fdtd_cop_s {
    // Device axes: the kernels' grid is the operator's with its axes
    // relabelled cyclically, device axis a = reference axis (a + rot) % 3
    // (and device component n = reference component (n + rot) % 3); every
    // array below is in device axes.  N0 is the operator's own grid.
    uint32_t N[3] = {0, 0, 0};
    uint32_t N0[3] = {0, 0, 0};
    int rot = 0;
    int Nzp = 0;
    long long comp = 0;
    double dT = 0;
    wipems::HalfTables E, H;
    bool geo = false;                  // factorized geometry (graded mesh)
    std::vector<float> geom;           // [4][Nx+Ny+Nz]: dE, iD, dH, iM per axis
    uint32_t upml_nodes = 0, ade_nodes = 0;
    int inner_lo[3] = {0, 0, 0}, inner_hi[3] = {0, 0, 0};  // nodes outside may be UPML
    bool trim_e[3] = {false, false, false};  // last line inert for the voltage update
    std::vector<float> sigV, sigC;
    std::vector<wipems::MurFace> mur;  // Mur ABC faces (copied from the operator)
    wipems::RlcList rlc;               // lumped RLC edges (copied from the operator)
    std::vector<double> edges;         // [2][Nx+Ny+Nz]: main / dual edge lengths in m (field dumps);
                                       // empty when the description has no mesh lines
    uint32_t sig_len = 0, sig_period = 0;
    ~fdtd_cop_s();
};
