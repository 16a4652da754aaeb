// Direct-load half-step kernels (fallback variant), the probe / energy
// reductions and the timestep counter.  The per-node arithmetic lives in
// node.cuh; the TMA-pipelined variant of the two half-step kernels is in
// kernels_tma.cuh.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "node.cuh"

namespace wipems {

// --------------------------------------------------------------- E half-step
// Block: 32 (z) x TY (y) threads, marching over x in [x0, x0+XC).  Shared
// memory double buffer: 3 components x (TY+1) rows x 33 cols; row 0 is the
// y-1 halo, column 0 the z-1 halo.
template <typename IdxT, int FEAT, bool GEO>
__global__ void __launch_bounds__(256) k_volt(const DevGrid g, int ts_off, int XC) {
    if (*g.d_done) return;
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
            const uint32_t t = load_idx<IdxT>(g.e.idx, o);
            float v[3] = {g.V[o], g.V[C + o], g.V[2 * C + o]};
            GeoF gf;
            if (GEO) gf = geo_factors(g, false, x, y, z);
            update_node<false, FEAT, GEO>(g, v, curl, t, o, numTS, nullptr, 0, gf);
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
template <typename IdxT, int FEAT, bool GEO, bool ENERGY>
__global__ void __launch_bounds__(256) k_curr(const DevGrid g, int ts_off, int XC) {
    if (*g.d_done) return;
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
        float eh[3] = {0.f, 0.f, 0.f};  // new I of this node (energy terms)
        if (active) {
            const float v2yp = s2[si + 33];
            const float v0yp = s0[si + 33];
            const float v1zp = s1[si + 1];
            const float v0zp = s0[si + 1];
            float curl[3];
            curl[0] = __fadd_rn(__fsub_rn(__fsub_rn(c2, v2yp), c1), v1zp);
            curl[1] = __fadd_rn(__fsub_rn(__fsub_rn(c0, v0zp), c2), n2);
            curl[2] = __fadd_rn(__fsub_rn(__fsub_rn(c1, n1), c0), v0yp);
            const uint32_t t = load_idx<IdxT>(g.h.idx, o);
            float cu[3] = {g.I[o], g.I[C + o], g.I[2 * C + o]};
            GeoF gf;
            if (GEO) gf = geo_factors(g, true, x, y, z);
            update_node<true, FEAT, GEO>(g, cu, curl, t, o, numTS, nullptr, 0, gf);
            g.I[o] = cu[0];
            g.I[C + o] = cu[1];
            g.I[2 * C + o] = cu[2];
            eh[0] = cu[0];
            eh[1] = cu[1];
            eh[2] = cu[2];
        }
        if (ENERGY)  // Engine_Interface_FDTD::CalcFastEnergy terms of segment (x, y, blockIdx.x)
            energy_segment(g, x, y, blockIdx.x, active, y < g.Ny - 1 && (int)blockIdx.x * 32 < g.Nz - 1, c0, c1, c2,
                           eh[0], eh[1], eh[2]);
        c0 = n0;
        c1 = n1;
        c2 = n2;
    }
}

// ---------------------------------------------------------- probes / counter
struct ProbeEntry {
    long long off;  // linear offset within the component (padded layout; grids may exceed 2^32 nodes)
    int8_t comp;    // 0..2
    int8_t sign;    // +1 / -1
    int8_t field;   // 0 = voltage, 1 = current
    int8_t pad[5];
};

struct ProbeSet {
    const ProbeEntry* entries;  // all probes' entries, concatenated
    const int* first;           // [nprobe+1] entry ranges
    const double* weight;       // [nprobe]
    const double* div;          // [nprobe]: 0 = an integral; > 0 = a field-probe column, value / div
                                // (the edge length); < 0 = a field-probe column on an edge of length 0
    int nprobe;
    int row_doubles;            // doubles per record row (2 + nprobe)
    double* ring;               // [cap][row_doubles]: ts, energy, values...
    int cap;
    int* d_nsamp;               // samples written
    int* d_err;                 // error word (ring overflow, non-finite)
    int* d_done;                // end criterion met (0 / 1)
    double end_crit;            // > 0: stop once energy <= end_crit * max energy
    int stop_ts;                // > 0 (with end_crit): stop at this numTS
};

// Integral of probe p over the fields of numTS ts, by one warp: the lanes
// load 32 entries at a time and the sum runs over them in entry order --
// the reference's own order and precision: ProcessVoltage's line sum in
// double (engine_interface_fdtd.cpp:200-226), ProcessCurrent's loop sum in
// float (processcurrent.cpp:93-168) -- so the samples are bit-identical to
// the reference's.  Every lane returns the sum.
__device__ __forceinline__ double probe_sum(const ProbeSet& ps, const DevGrid& g, int p, int ts, int lane) {
    const int first = ps.first[p], last = ps.first[p + 1];
    if (first >= last) return 0.0;
    const bool odd = g.V2 && (ts & 1);  // fused kernel: the buffer of numTS
    const bool current = ps.entries[first].field != 0;
    double accd = 0.0;
    float accf = 0.f;
    for (int base = first; base < last; base += 32) {
        float v = 0.f;
        int sg = 1;
        if (base + lane < last) {
            const ProbeEntry pe = ps.entries[base + lane];
            const float* f = pe.field ? (odd ? g.I2 : g.I) : (odd ? g.V2 : g.V);
            v = f[(long long)pe.comp * g.comp + pe.off];
            sg = pe.sign;
        }
        const int cnt = min(32, last - base);
        for (int k = 0; k < cnt; ++k) {
            const float vk = __shfl_sync(0xffffffffu, v, k);
            const int sk = __shfl_sync(0xffffffffu, sg, k);
            if (current) accf = sk > 0 ? __fadd_rn(accf, vk) : __fsub_rn(accf, vk);
            else accd = sk > 0 ? __dadd_rn(accd, (double)vk) : __dsub_rn(accd, (double)vk);
        }
    }
    return current ? (double)accf : accd;
}

// Sample column p: an integral (probe_sum) or one component of a field
// probe, GetRawField / GetRawDualField (engine_interface_fdtd.cpp:257-266
// and 128-142): the field value in double divided by the edge length, 0 for
// an edge of length 0.
__device__ __forceinline__ double probe_value(const ProbeSet& ps, const DevGrid& g, int p, int ts, int lane) {
    const double dv = ps.div[p];
    if (dv == 0.0) return probe_sum(ps, g, p, ts, lane);
    if (dv < 0.0) return 0.0;
    const ProbeEntry pe = ps.entries[ps.first[p]];
    const bool odd = g.V2 && (ts & 1);
    const float* f = pe.field ? (odd ? g.I2 : g.I) : (odd ? g.V2 : g.V);
    return (double)f[(long long)pe.comp * g.comp + pe.off] / dv;
}

// Frequency-domain probe accumulation (ProcessIntegral::Process,
// processintegral.cpp:154-168): on every FD step, for each probe p and
// frequency f,  F[p][f] += v_p * weight_p * exp(-2 pi i f t_p) * scale  with
// t_p = (numTS + 0.5 for current probes) * dT and scale = 2 dT FD_interval.
struct FdSet {
    int nfreq;
    const double* freq;  // [nfreq] Hz
    double* acc;         // [nprobe][nfreq][2] re, im
    const int* dual;     // [nprobe] 1: sampled at the dual time (current probe)
    double dT;
    double scale;
    int* count;          // FD samples accumulated
};

// One block; dynamic shared memory: nprobe doubles.  expect_ts: the numTS
// the host launched this for (a job that stopped on its end criterion
// earlier has a smaller numTS and is left alone).
static __global__ void k_fd_accumulate(const int* d_ts, int expect_ts, ProbeSet ps, const DevGrid g, FdSet fd) {
    extern __shared__ double s_val[];
    __shared__ int s_go;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
    if (tid == 0) s_go = (*d_ts == expect_ts);
    __syncthreads();
    if (!s_go) return;
    for (int p = warp; p < ps.nprobe; p += nwarps) {
        const double acc = probe_value(ps, g, p, expect_ts, lane);
        if (lane == 0) s_val[p] = acc * ps.weight[p];
    }
    __syncthreads();
    const int n = ps.nprobe * fd.nfreq;
    for (int k = tid; k < n; k += blockDim.x) {
        const int p = k / fd.nfreq, f = k - p * fd.nfreq;
        const double t = ((double)expect_ts + 0.5 * (double)fd.dual[p]) * fd.dT;
        double sn, cs;
        sincospi(2.0 * fd.freq[f] * t, &sn, &cs);  // exp(-2 pi i f t) = cs - i sn
        const double v = s_val[p] * fd.scale;
        fd.acc[2 * k] += v * cs;
        fd.acc[2 * k + 1] -= v * sn;
    }
    if (tid == 0) *fd.count += 1;
}

// Advances numTS by adv (Engine::IterateTS ++numTS) and, when sample is set,
// records one probe/energy sample row (ProcessIntegral::Process): the probe
// sums (ProcessVoltage / ProcessCurrent) as warp reductions in double.
// With an end criterion the job stops here, on the device, the way
// openEMS::RunFDTD's loop ends (openems.cpp:1285-1314): at the first sample
// whose energy is <= end_crit times the largest energy seen so far, or at
// stop_ts timesteps; a stopped job's kernels and samplers do nothing.
// tid / nthr: the calling thread's linear index in the block and the
// block's thread count (a multiple of 32); every thread of the block calls.
__device__ __forceinline__ void advance_sample(int* d_ts, int adv, int sample, const ProbeSet& ps, const DevGrid& g,
                                               int energy_valid, double eps0, double mue0, int tid, int nthr) {
    __shared__ int s_ts, s_row, s_done;
    if (tid == 0) {
        s_row = -1;
        s_done = *ps.d_done;
    }
    __syncthreads();
    if (s_done) return;
    if (tid == 0) {
        int ts = *d_ts + adv;
        if (adv) *d_ts = ts;
        s_ts = ts;
        if (ps.end_crit > 0.0 && ps.stop_ts > 0 && ts >= ps.stop_ts) *ps.d_done = 1;
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
    const int warp = tid >> 5, lane = tid & 31;
    const int nwarps = nthr >> 5;
    for (int p = warp; p < ps.nprobe; p += nwarps) {
        const double acc = probe_value(ps, g, p, s_ts, lane);
        if (lane == 0) rec[2 + p] = acc * ps.weight[p];
    }
    if (tid == 0) {
        rec[0] = (double)s_ts;
        if (energy_valid) {
            // the plane sums in x order (fixed by the grid)
            double a = 0.0, b = 0.0;
            for (int x = 0; x < g.Nx - 1; ++x) {
                const double2 p = g.eplane[x];
                a += p.x;
                b += p.y;
            }
            double e = eps0 * a + mue0 * b;
            if (!isfinite(e)) atomicOr(ps.d_err, 2);
            rec[1] = e;
            if (ps.end_crit > 0.0) {
                const double m = fmax(g.d_eacc[2], e);
                g.d_eacc[2] = m;
                if (m > 0.0 && e / m <= ps.end_crit) *ps.d_done = 1;
            }
        } else {
            rec[1] = -1.0;
        }
    }
}

// Sum of the energy segments of plane x in a fixed order (256 threads: each
// sums a strided share in double, then a fixed shuffle / shared-memory
// tree); thread 0 returns the pair.
__device__ __forceinline__ double2 plane_energy(const DevGrid& g, int x) {
    __shared__ double sa[8], sb[8];
    const long long n = (long long)(g.Ny - 1) * g.nzt;
    const float2* seg = g.eseg + (long long)x * n;
    double a = 0.0, b = 0.0;
    for (long long i = threadIdx.x; i < n; i += 256) {
        const float2 v = seg[i];
        a += (double)v.x;
        b += (double)v.y;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, off);
        b += __shfl_down_sync(0xffffffffu, b, off);
    }
    if ((threadIdx.x & 31) == 0) {
        sa[threadIdx.x >> 5] = a;
        sb[threadIdx.x >> 5] = b;
    }
    __syncthreads();
    double2 r = make_double2(0.0, 0.0);
    if (threadIdx.x == 0) {
        for (int w = 0; w < 8; ++w) {
            r.x += sa[w];
            r.y += sb[w];
        }
    }
    return r;
}

// one probe integral of the current fields (one warp), written to out[0]
static __global__ void k_probe_now(ProbeSet ps, const DevGrid g, double* out) {
    const double v = probe_value(ps, g, 0, 0, threadIdx.x & 31);
    if (threadIdx.x == 0) out[0] = v;
}

// one block (256 threads) per x plane: eplane[x] from the plane's segments
static __global__ void __launch_bounds__(256) k_energy_planes(const DevGrid g) {
    const double2 r = plane_energy(g, blockIdx.x);
    if (threadIdx.x == 0) g.eplane[blockIdx.x] = r;
}

static __global__ void k_advance_sample(int* d_ts, int adv, int sample, ProbeSet ps, const DevGrid g, int energy_valid,
                                        double eps0, double mue0) {
    advance_sample(d_ts, adv, sample, ps, g, energy_valid, eps0, mue0, threadIdx.x, blockDim.x);
}

// ------------------------------------------------------------- Mur ABC
// Engine_Ext_Mur_ABC (engine_ext_mur_abc.cpp:84-164) on the device, three
// passes around the voltage kernel: stage 0 (before it, old V):
// b = V(shift) - c V(line); stage 1 (after it): b += c V(shift); stage 2:
// V(line) = b, then the line node's own excitation, if any (the reference
// adds excitations after every other voltage hook).  Faces are in face
// order (xmin .. zmax); where two faces share a node component the one
// earlier in that order writes it, as the reference applies them in
// reverse insertion order.  A face acts from numTS >= start_ts on.
struct MurDev {
    int ny, line, shift, n0, n1, start_ts;
    const float* cp;
    const float* cpp;
    float* bp;
    float* bpp;
    uint32_t offset;  // first flattened index of this face in the launch
};
struct MurSet {
    int nface;
    int idx16;        // E tuple index width (for the excitation lookup)
    int trim[3];      // the last line of this axis is left out of the voltage kernel (inert)
    uint32_t total;
    MurDev f[6];
};

static __global__ void k_mur(const DevGrid g, MurSet ms, int ts_off, int stage) {
    if (*g.d_done) return;
    const int numTS = *g.d_ts + ts_off;
    const long long C = g.comp;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < ms.total; k += gridDim.x * blockDim.x) {
        int fi = 0;
        while (fi + 1 < ms.nface && k >= ms.f[fi + 1].offset) ++fi;
        const MurDev& F = ms.f[fi];
        if (numTS < F.start_ts) continue;
        const uint32_t loc = k - F.offset;
        const int i = (int)(loc / (uint32_t)F.n1), j = (int)(loc - (uint32_t)i * (uint32_t)F.n1);
        const int ny = F.ny, nP = (ny + 1) % 3, nPP = (ny + 2) % 3;
        int pos[3], sh[3];
        pos[ny] = F.line;
        sh[ny] = F.shift;
        pos[nP] = sh[nP] = i;
        pos[nPP] = sh[nPP] = j;
        const long long ol = (long long)pos[0] * g.sx + (long long)pos[1] * g.Nzp + pos[2];
        const long long os = (long long)sh[0] * g.sx + (long long)sh[1] * g.Nzp + sh[2];
        float* V = g.V;
        if (stage == 0) {
            F.bp[loc] = __fsub_rn(V[nP * C + os], __fmul_rn(F.cp[loc], V[nP * C + ol]));
            F.bpp[loc] = __fsub_rn(V[nPP * C + os], __fmul_rn(F.cpp[loc], V[nPP * C + ol]));
        } else if (stage == 1) {
            // on a last line the voltage kernel leaves out (all its edges inert)
            // the update's result is zero: read that instead of the value an
            // earlier apply left there
            const bool inert = (ms.trim[nP] && sh[nP] == (nP == 0 ? g.Nx : nP == 1 ? g.Ny : g.Nz) - 1) ||
                               (ms.trim[nPP] && sh[nPP] == (nPP == 0 ? g.Nx : nPP == 1 ? g.Ny : g.Nz) - 1);
            const float vP = inert ? 0.f : V[nP * C + os];
            const float vPP = inert ? 0.f : V[nPP * C + os];
            F.bp[loc] = __fadd_rn(F.bp[loc], __fmul_rn(F.cp[loc], vP));
            F.bpp[loc] = __fadd_rn(F.bpp[loc], __fmul_rn(F.cpp[loc], vPP));
        } else {
            const int comps[2] = {nP, nPP};
            const float vals[2] = {F.bp[loc], F.bpp[loc]};
            uint32_t t = 0;
            uint32_t flags = 0;
            bool have_t = false;
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                const int c = comps[q];
                bool mine = true;  // an earlier active face sharing this component writes it
                for (int e = 0; e < fi; ++e) {
                    const MurDev& G = ms.f[e];
                    if (numTS >= G.start_ts && pos[G.ny] == G.line && c != G.ny) mine = false;
                }
                if (!mine) continue;
                float v = vals[q];
                if (!have_t) {
                    t = ms.idx16 ? load_idx<uint16_t>(g.e.idx, ol) : load_idx<uint32_t>(g.e.idx, ol);
                    flags = __float_as_uint(__ldg(&g.e.main[TAB_MAIN * t + 1]).z);
                    have_t = true;
                }
                if (flags & TF_EXC) {
                    const float4 e0 = __ldg(&g.e.exc[TAB_EXC * t]);
                    const float4 e1 = __ldg(&g.e.exc[TAB_EXC * t + 1]);
                    const float amp[3] = {e0.x, e0.y, e0.z};
                    const int dly[3] = {__float_as_int(e1.x), __float_as_int(e1.y), __float_as_int(e1.z)};
                    if (dly[c] >= 0) {
                        const int kx = exc_index(numTS, dly[c], g.sig_len, g.sig_period);
                        v = __fadd_rn(v, __fmul_rn(amp[c], g.sigV[kx]));
                    }
                }
                V[c * C + ol] = v;
            }
        }
    }
}

// ------------------------------------------------------------- lumped RLC
// Engine_Ext_LumpedRLC (engine_ext_lumpedRLC.cpp:83-145) on the device: one
// pass after the voltage kernel (and after the Mur post-update, before the
// Mur apply), one thread per RLC edge.  The reference rotates its Vd[0..2]
// and J[0..2] buffers every step; here the history is a ring indexed by
// numTS: slot numTS % 3 is [n], (numTS + 2) % 3 is [n-1], (numTS + 1) % 3
// is [n-2].  The pre-update (parallel inductor current) touches only the
// element's own state, so it runs in the same pass.  Float products and
// sums in the reference's order.
struct RlcSet {
    uint32_t count;
    const long long* off;  // dir * comp + x * sx + y * Nzp + z
    const float* coef;     // [9][count]: ilv, i2v, vv2, vj1, vj2, vvd, ib0, b1, b2
    float* state;          // [7][count]: Il, Vd[3 slots], J[3 slots]
};

static __global__ void k_rlc(const DevGrid g, RlcSet rs, int ts_off) {
    if (*g.d_done) return;
    const int numTS = *g.d_ts + ts_off;
    const uint32_t n = rs.count;
    const uint32_t s0 = (uint32_t)(numTS % 3), s1 = (uint32_t)((numTS + 2) % 3), s2 = (uint32_t)((numTS + 1) % 3);
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const float* c = rs.coef + k;
        const float ilv = c[0], i2v = c[n], vv2 = c[2 * n], vj1 = c[3 * n], vj2 = c[4 * n], vvd = c[5 * n],
                    ib0 = c[6 * n], b1 = c[7 * n], b2 = c[8 * n];
        float* Il = rs.state + k;
        float* Vd = rs.state + n + k;
        float* J = rs.state + 4 * n + k;
        // DoPreVoltageUpdates: Il += i2v * ilv * Vd[n-1]
        const float il = __fadd_rn(Il[0], __fmul_rn(__fmul_rn(i2v, ilv), Vd[s1 * n]));
        Il[0] = il;
        const float vd2 = Vd[s2 * n], j1 = J[s1 * n], j2 = J[s2 * n];
        // Apply2Voltages
        float t = __fsub_rn(g.V[rs.off[k]], il);
        t = __fadd_rn(t, __fmul_rn(vv2, vd2));
        t = __fadd_rn(t, __fmul_rn(vj1, j1));
        t = __fadd_rn(t, __fmul_rn(vj2, j2));
        const float vd = __fmul_rn(vvd, t);
        float jn = __fmul_rn(ib0, __fsub_rn(vd, vd2));
        jn = __fsub_rn(jn, __fmul_rn(__fmul_rn(b1, ib0), j1));
        jn = __fsub_rn(jn, __fmul_rn(__fmul_rn(b2, ib0), j2));
        Vd[s0 * n] = vd;
        J[s0 * n] = jn;
        g.V[rs.off[k]] = vd;
    }
}

// ------------------------------------------------------------- field dumps
// ProcessFields::CalcField (processfields.cpp:280-330) for E and H dumps on
// the device: Engine_Interface_FDTD::GetRawInterpolatedField /
// GetRawInterpolatedDualField (engine_interface_fdtd.cpp:60-200) with
// GetRawField / GetRawDualField (E = V / edge length, H = I / dual edge
// length, 0 where the length is 0), in double and in the reference's order,
// stored as float like the reference's FDTD_FLOAT field arrays.  Output
// [3][n0][n1][n2] at the mesh lines start + i * step.
struct DumpBox {
    int field;   // 0 = E, 1 = H
    int interp;  // 0 = none, 1 = node, 2 = cell
    int start[3], step[3], num[3];
};

static __global__ void k_dump_field(const DevGrid g, const float* __restrict__ V, const float* __restrict__ I,
                                    const double* __restrict__ edges, DumpBox b, float* __restrict__ out) {
    const long long total = (long long)b.num[0] * b.num[1] * b.num[2];
    const int Nn[3] = {g.Nx, g.Ny, g.Nz};
    const int eoff[3] = {0, g.Nx, g.Nx + g.Ny};
    const int ntot = g.Nx + g.Ny + g.Nz;
    auto len = [&](int n, int p, bool dual) -> double { return edges[(dual ? ntot : 0) + eoff[n] + p]; };
    auto at = [&](int n, const int* p) -> long long {
        return n * g.comp + (long long)p[0] * g.sx + (long long)p[1] * g.Nzp + p[2];
    };
    auto rawE = [&](int n, const int* p) -> double {  // GetRawField, type 0
        const double value = V[at(n, p)];
        const double delta = len(n, p[n], false);
        return delta != 0.0 ? value / delta : 0.0;
    };
    auto rawH = [&](int n, const int* p) -> double {  // GetRawDualField, type 0
        const double value = I[at(n, p)];
        const double delta = len(n, p[n], true);
        return delta != 0.0 ? value / delta : 0.0;
    };
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < total;
         k += (long long)gridDim.x * blockDim.x) {
        const int l = (int)(k % b.num[2]);
        const int j = (int)((k / b.num[2]) % b.num[1]);
        const int i = (int)(k / ((long long)b.num[1] * b.num[2]));
        const int pos[3] = {b.start[0] + i * b.step[0], b.start[1] + j * b.step[1], b.start[2] + l * b.step[2]};
        int q[3] = {pos[0], pos[1], pos[2]};
        double o[3];
        const bool top = pos[0] == Nn[0] - 1 || pos[1] == Nn[1] - 1 || pos[2] == Nn[2] - 1;
        for (int n = 0; n < 3; ++n) {
            const int nP = (n + 1) % 3, nPP = (n + 2) % 3;
            if (b.field == 0) {
                if (b.interp == 0) {
                    o[n] = rawE(n, pos);
                } else if (b.interp == 1) {  // node: edge-length weighted mean of the two edges at the node
                    if (pos[n] == Nn[n] - 1) {
                        --q[n];
                        o[n] = rawE(n, q);
                        ++q[n];
                        continue;
                    }
                    const double delta = len(n, q[n], false);
                    o[n] = rawE(n, q);
                    if (delta == 0.0) {
                        o[n] = 0.0;
                        continue;
                    }
                    if (pos[n] == 0) continue;
                    --q[n];
                    const double deltaDown = len(n, q[n], false);
                    const double deltaRel = delta / (delta + deltaDown);
                    o[n] = o[n] * (1.0 - deltaRel) + rawE(n, q) * deltaRel;
                    ++q[n];
                } else {  // cell: mean of the four edges around the cell centre line
                    if (top) {
                        o[n] = 0.0;
                        continue;
                    }
                    o[n] = rawE(n, q);
                    ++q[nP];
                    o[n] += rawE(n, q);
                    ++q[nPP];
                    o[n] += rawE(n, q);
                    --q[nP];
                    o[n] += rawE(n, q);
                    --q[nPP];
                    o[n] /= 4;
                }
            } else {
                if (b.interp == 0) {
                    o[n] = rawH(n, pos);
                } else if (b.interp == 1) {  // node: mean of the four dual edges around the node
                    if (top || pos[nP] == 0 || pos[nPP] == 0) {
                        o[n] = 0.0;
                        continue;
                    }
                    o[n] = rawH(n, q);
                    --q[nP];
                    o[n] += rawH(n, q);
                    --q[nPP];
                    o[n] += rawH(n, q);
                    ++q[nP];
                    o[n] += rawH(n, q);
                    ++q[nPP];
                    o[n] /= 4;
                } else {  // cell: dual-length weighted mean along n
                    const double delta = len(n, q[n], true);
                    o[n] = rawH(n, q);
                    if (pos[n] >= Nn[n] - 1) {
                        o[n] = 0.0;
                        continue;
                    }
                    ++q[n];
                    const double deltaUp = len(n, q[n], true);
                    const double deltaRel = delta / (delta + deltaUp);
                    o[n] = o[n] * (1.0 - deltaRel) + rawH(n, q) * deltaRel;
                    --q[n];
                }
            }
        }
        for (int n = 0; n < 3; ++n) out[n * total + k] = (float)o[n];
    }
}

// Full-grid energy (CalcFastEnergy) on demand: the segments from the fields
// with the same per-node terms and the same warp tree as the current
// kernels, so that (with k_energy_planes and k_energy_total) the result is
// bit-identical to the energy a sample step records for the same fields.
// Blocks of (32 z, 8 y) at one x plane (blockIdx.z).
static __global__ void k_energy_segments(const DevGrid g) {
    const int x = blockIdx.z, y = blockIdx.y * 8 + threadIdx.y, zt = blockIdx.x;
    const int z = zt * 32 + threadIdx.x;
    const bool act = (y < g.Ny - 1) && (z < g.Nz - 1);
    float v[3] = {0.f, 0.f, 0.f}, c[3] = {0.f, 0.f, 0.f};
    if (act) {
        const long long o = (long long)x * g.sx + (long long)y * g.Nzp + z;
#pragma unroll
        for (int n = 0; n < 3; ++n) {
            v[n] = g.V[n * g.comp + o];
            c[n] = g.I[n * g.comp + o];
        }
    }
    energy_segment(g, x, y, zt, act, y < g.Ny - 1, v[0], v[1], v[2], c[0], c[1], c[2]);
}

// eps0 * sum E + mue0 * sum H over the planes in x order (one thread)
static __global__ void k_energy_total(const DevGrid g, double eps0, double mue0, double* out) {
    if (threadIdx.x != 0) return;
    double a = 0.0, b = 0.0;
    for (int x = 0; x < g.Nx - 1; ++x) {
        const double2 p = g.eplane[x];
        a += p.x;
        b += p.y;
    }
    out[0] = eps0 * a + mue0 * b;
}

}  // namespace wipems
