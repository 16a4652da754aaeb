// Batched mode: many independent simulations of uneven grid sizes advance
// together, one persistent kernel per half-step (per kernel variant) over a
// flattened (job, tile, x-chunk) work list, with every job's probes and
// energy sampled on the device at its own probe interval.  The timestep
// sequence [voltage kernels, current kernels, sampler] is captured into a
// CUDA graph and replayed.
//
// A job is an ordinary engine (fdtd_engine_create*): the batch only refers
// to its device arrays, so per-job calls (read_samples, get_fields, reset)
// keep working between batch iterations.  Jobs of different kernel variants
// (uint16 / uint32 tuple index, UPML / ADE features, factorized geometry)
// form separate groups, each with its own persistent kernels; the groups of
// one half-step run concurrently.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "engine_state.h"

namespace wipems {
namespace {

// per-job state of the batched sampler
struct AdvJob {
    int* d_ts;
    ProbeSet ps;
    DevGrid g;
    int interval;
    int energy_valid;
    const int* ctl;  // the job's control words (numTS, samples, errors, done)
    int* out;        // the batch's copy of them, read back after each iterate
};

// Block j advances job j's numTS by one and records a sample row when the
// new timestep is a multiple of the job's probe interval (the decision is
// taken on the device, so the step sequence can be replayed as a graph).
__global__ void k_batch_advance(const AdvJob* __restrict__ jobs, double eps0, double mue0) {
    const AdvJob& J = jobs[blockIdx.x];
    const int ts = *J.d_ts + 1;
    const int sample = (J.interval > 0 && (ts % J.interval) == 0) ? 1 : 0;
    advance_sample(J.d_ts, 1, sample, J.ps, J.g, J.energy_valid, eps0, mue0, threadIdx.x, blockDim.x);
    __syncthreads();
    if (threadIdx.x < 4) J.out[threadIdx.x] = J.ctl[threadIdx.x];
}

// Energy plane sums (k_energy_planes) of the jobs that record a sample
// after this step: block (x, j) sums plane x of job j (the same fixed order
// as a job running alone, so its energies are the same bits).
__global__ void __launch_bounds__(256) k_batch_energy_planes(const AdvJob* __restrict__ jobs) {
    const AdvJob& J = jobs[blockIdx.y];
    if (!J.energy_valid || J.interval <= 0 || *J.g.d_done) return;
    if ((*J.d_ts + 1) % J.interval != 0 || (int)blockIdx.x >= J.g.Nx - 1) return;
    const double2 r = plane_energy(J.g, (int)blockIdx.x);
    if (threadIdx.x == 0) J.g.eplane[blockIdx.x] = r;
}

// The jobs of one kernel variant (index width, features, geometry mode) in
// one bin, or one chain's share of them: a contiguous range of the batch's
// job order, so the range's samplers are one launch.
struct Group {
    int bin = 0;
    bool e16 = true, h16 = true, geo = false;
    int feat = 0;    // the voltage kernel's feature set
    int feat_h = 0;  // the current kernel's
    std::vector<int> jobs;
    DevBuf<WorkItem> itE, itH;
    int nE = 0, nH = 0, gridE = 0, gridH = 0;
    size_t smemE = 0, smemH = 0;
    int first = 0, count = 0;  // job range
    int max_planes = 1;        // largest Nx-1 of its jobs
};

// The batched kernels come in two tile heights (TY rows of 32 z-lanes per
// block, the same rows in every job's tensor maps): 8 (256 threads) or 4.
template <typename IdxT, int FEAT, bool GEO, int TY>
void volt_batch_launch(const Group& G, const BatchJob* jobs, int XC, int S, cudaStream_t st) {
    k_volt_batch<IdxT, FEAT, GEO, TY><<<G.gridE, dim3(32, TY), G.smemE, st>>>(jobs, G.itE.p, G.nE, XC, S);
}
template <typename IdxT, int FEAT, bool GEO, int TY>
void curr_batch_launch(const Group& G, const BatchJob* jobs, int XC, int S, cudaStream_t st) {
    k_curr_batch<IdxT, FEAT, GEO, TY><<<G.gridH, dim3(32, TY), G.smemH, st>>>(jobs, G.itH.p, G.nH, XC, S);
}

template <typename IdxT, bool GEO, int TY>
void volt_feat(const Group& G, const BatchJob* jobs, int XC, int S, cudaStream_t st) {
    switch (G.feat) {
        case 0: volt_batch_launch<IdxT, 0, GEO, TY>(G, jobs, XC, S, st); break;
        case 1: volt_batch_launch<IdxT, 1, GEO, TY>(G, jobs, XC, S, st); break;
        case 2: volt_batch_launch<IdxT, 2, GEO, TY>(G, jobs, XC, S, st); break;
        default: volt_batch_launch<IdxT, 3, GEO, TY>(G, jobs, XC, S, st); break;
    }
}
template <typename IdxT, bool GEO, int TY>
void curr_feat(const Group& G, const BatchJob* jobs, int XC, int S, cudaStream_t st) {
    switch (G.feat_h) {
        case 0: curr_batch_launch<IdxT, 0, GEO, TY>(G, jobs, XC, S, st); break;
        case 1: curr_batch_launch<IdxT, 1, GEO, TY>(G, jobs, XC, S, st); break;
        case 2: curr_batch_launch<IdxT, 2, GEO, TY>(G, jobs, XC, S, st); break;
        default: curr_batch_launch<IdxT, 3, GEO, TY>(G, jobs, XC, S, st); break;
    }
}

template <int TY>
void group_volt_ty(const Group& G, const BatchJob* jobs, int XC, int S, cudaStream_t st) {
    if (G.e16) {
        if (G.geo) volt_feat<uint16_t, true, TY>(G, jobs, XC, S, st);
        else volt_feat<uint16_t, false, TY>(G, jobs, XC, S, st);
    } else {
        if (G.geo) volt_feat<uint32_t, true, TY>(G, jobs, XC, S, st);
        else volt_feat<uint32_t, false, TY>(G, jobs, XC, S, st);
    }
}
template <int TY>
void group_curr_ty(const Group& G, const BatchJob* jobs, int XC, int S, cudaStream_t st) {
    if (G.h16) {
        if (G.geo) curr_feat<uint16_t, true, TY>(G, jobs, XC, S, st);
        else curr_feat<uint16_t, false, TY>(G, jobs, XC, S, st);
    } else {
        if (G.geo) curr_feat<uint32_t, true, TY>(G, jobs, XC, S, st);
        else curr_feat<uint32_t, false, TY>(G, jobs, XC, S, st);
    }
}
void launch_group_volt(const Group& G, const BatchJob* jobs, int XC, int S, cudaStream_t st, int ty) {
    if (ty == 4) group_volt_ty<4>(G, jobs, XC, S, st);
    else group_volt_ty<8>(G, jobs, XC, S, st);
}
void launch_group_curr(const Group& G, const BatchJob* jobs, int XC, int S, cudaStream_t st, int ty) {
    if (ty == 4) group_curr_ty<4>(G, jobs, XC, S, st);
    else group_curr_ty<8>(G, jobs, XC, S, st);
}

// occupancy of one batched kernel variant (blocks per SM)
template <typename IdxT, int FEAT, bool GEO, int TY>
int occ_one(bool volt, size_t smem) {
    int n = 0;
    if (volt)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_volt_batch<IdxT, FEAT, GEO, TY>, 32 * TY, smem);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_curr_batch<IdxT, FEAT, GEO, TY>, 32 * TY, smem);
    return n;
}
template <typename IdxT, bool GEO, int TY>
int occ_feat(int feat, bool volt, size_t smem) {
    switch (feat) {
        case 0: return occ_one<IdxT, 0, GEO, TY>(volt, smem);
        case 1: return occ_one<IdxT, 1, GEO, TY>(volt, smem);
        case 2: return occ_one<IdxT, 2, GEO, TY>(volt, smem);
        default: return occ_one<IdxT, 3, GEO, TY>(volt, smem);
    }
}
template <int TY>
int occupancy_ty(const Group& G, bool volt, size_t smem) {
    const bool i16 = volt ? G.e16 : G.h16;
    if (i16)
        return G.geo ? occ_feat<uint16_t, true, TY>(volt ? G.feat : G.feat_h, volt, smem)
                     : occ_feat<uint16_t, false, TY>(volt ? G.feat : G.feat_h, volt, smem);
    return G.geo ? occ_feat<uint32_t, true, TY>(volt ? G.feat : G.feat_h, volt, smem)
                 : occ_feat<uint32_t, false, TY>(volt ? G.feat : G.feat_h, volt, smem);
}
int occupancy(const Group& G, bool volt, size_t smem, int ty) {
    return ty == 4 ? occupancy_ty<4>(G, volt, smem) : occupancy_ty<8>(G, volt, smem);
}

template <typename IdxT, int FEAT, bool GEO>
cudaError_t batch_smem_attr_one(int bytes) {
    const cudaFuncAttribute a = cudaFuncAttributeMaxDynamicSharedMemorySize;
    const cudaError_t r[4] = {cudaFuncSetAttribute(k_volt_batch<IdxT, FEAT, GEO, 8>, a, bytes),
                              cudaFuncSetAttribute(k_curr_batch<IdxT, FEAT, GEO, 8>, a, bytes),
                              cudaFuncSetAttribute(k_volt_batch<IdxT, FEAT, GEO, 4>, a, bytes),
                              cudaFuncSetAttribute(k_curr_batch<IdxT, FEAT, GEO, 4>, a, bytes)};
    for (cudaError_t x : r)
        if (x != cudaSuccess) return x;
    return cudaSuccess;
}

int batch_smem_attrs(int bytes) {
    cudaError_t r = cudaSuccess, t;
#define WIPEMS_BATTR(I, F)                                                     \
    if ((t = batch_smem_attr_one<I, F, false>(bytes)) != cudaSuccess) r = t;   \
    if ((t = batch_smem_attr_one<I, F, true>(bytes)) != cudaSuccess) r = t;
    WIPEMS_BATTR(uint16_t, 0) WIPEMS_BATTR(uint16_t, 1) WIPEMS_BATTR(uint16_t, 2) WIPEMS_BATTR(uint16_t, 3)
    WIPEMS_BATTR(uint32_t, 0) WIPEMS_BATTR(uint32_t, 1) WIPEMS_BATTR(uint32_t, 2) WIPEMS_BATTR(uint32_t, 3)
#undef WIPEMS_BATTR
    if (r != cudaSuccess) {
        set_error(std::string("cudaFuncSetAttribute (batch): ") + cudaGetErrorString(r));
        return FDTD_ERR_CUDA;
    }
    return FDTD_OK;
}

// Why an engine cannot join a batch (0 = it can; the message is set).
int batch_refusal(const fdtd_engine_s* e) {
    if (!e->use_tma || e->fused) {
        set_error("fdtd_batch_create: jobs must use the two-pass TMA kernels");
        return FDTD_ERR_ARG;
    }
    if (e->mur.nface) {
        set_error("fdtd_batch_create: Mur boundaries are not provided in batches");
        return FDTD_ERR_UNSUPPORTED;
    }
    if (e->rlc.count) {
        set_error("fdtd_batch_create: lumped RLC elements are not provided in batches");
        return FDTD_ERR_UNSUPPORTED;
    }
    if (e->fd_interval) {
        set_error("fdtd_batch_create: frequency-domain accumulation is not provided in batches");
        return FDTD_ERR_UNSUPPORTED;
    }
    if (e->feat & FEAT_ADEX) {
        set_error("fdtd_batch_create: Lorentz/Drude dispersion of order > 1 is not provided in batches");
        return FDTD_ERR_UNSUPPORTED;
    }
    return FDTD_OK;
}

template <int T>
size_t stage_smem_ty(bool i16, bool upml, bool ade, int S) {
    if (ade) {  // voltage kernels of groups with Lorentz/Drude nodes stage their states too
        if (i16)
            return upml ? StageLayout<uint16_t, true, true, T>::smem(S) : StageLayout<uint16_t, false, true, T>::smem(S);
        return upml ? StageLayout<uint32_t, true, true, T>::smem(S) : StageLayout<uint32_t, false, true, T>::smem(S);
    }
    if (i16) return upml ? StageLayout<uint16_t, true, false, T>::smem(S) : StageLayout<uint16_t, false, false, T>::smem(S);
    return upml ? StageLayout<uint32_t, true, false, T>::smem(S) : StageLayout<uint32_t, false, false, T>::smem(S);
}
size_t stage_smem(bool i16, bool upml, bool ade, int S, int ty) {  // the batched kernels' stages
    return ty == 4 ? stage_smem_ty<4>(i16, upml, ade, S) : stage_smem_ty<8>(i16, upml, ade, S);
}

}  // namespace
}  // namespace wipems

using namespace wipems;

struct fdtd_batch_s {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<fdtd_engine_s*> jobs;
    std::vector<Group> groups;
    DevBuf<BatchJob> d_jobs;
    DevBuf<TmaMaps> d_maps;
    DevBuf<AdvJob> d_adv;
    DevBuf<int> d_status;      // [jobs][4] control words of every job
    std::vector<int> h_status;
    // L2 bins: jobs whose footprints together fit a bin run graph_steps
    // steps in a row while their data stays in L2, then the next bin runs
    struct Bin {
        std::vector<int> groups;
        int first = 0, count = 0;  // job range (jobs are stored bin by bin)
        int max_planes = 1;        // largest Nx-1 of the bin's jobs
    };
    std::vector<Bin> bins;
    uint64_t bin_bytes = 0;
    int XC = 8, stages = 3, blocks_per_sm = 0;
    int chains = 1;                    // chains per kernel-variant group
    int ty = BATCH_TY;                 // tile rows of the batched kernels (4 or 8)
    std::vector<cudaStream_t> side;    // one stream per chain of a bin
    std::vector<cudaEvent_t> ev_fork, ev_join;
    uint32_t graph_steps = 8;
    cudaGraphExec_t graph = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    double last_ms = 0;
    uint64_t last_launches = 0;
    uint64_t device_bytes = 0;
    uint64_t total_nodes = 0;
    ~fdtd_batch_s() {
        if (graph) cudaGraphExecDestroy(graph);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        for (cudaEvent_t e : ev_fork) cudaEventDestroy(e);
        for (cudaEvent_t e : ev_join) cudaEventDestroy(e);
        for (cudaStream_t s : side) cudaStreamDestroy(s);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace wipems {
namespace {

// one timestep of the jobs of bin k: the voltage kernels of the bin's
// groups, their current kernels, then the bin's samplers.  (Running the
// groups of a half-step concurrently on side streams was measured slower:
// each persistent grid already fills the GPU.)
// one timestep of chain G (a group's job range) on stream st: its voltage
// kernel, its current kernel, then the samplers of its jobs
void chain_step(fdtd_batch_s* b, const Group& G, cudaStream_t st) {
    launch_group_volt(G, b->d_jobs.p, b->XC, b->stages, st, b->ty);
    launch_group_curr(G, b->d_jobs.p, b->XC, b->stages, st, b->ty);
    k_batch_energy_planes<<<dim3((unsigned)G.max_planes, (unsigned)G.count), 256, 0, st>>>(b->d_adv.p + G.first);
    k_batch_advance<<<(unsigned)G.count, 256, 0, st>>>(b->d_adv.p + G.first, kEps0, kMue0);
    b->last_launches += 4;
}

// `steps` timesteps of bin k as independent chains: fork the chains' streams
// off the batch stream, run each chain's steps on its own stream, join
int bin_chains(fdtd_batch_s* b, size_t k, uint32_t steps) {
    const fdtd_batch_s::Bin& B = b->bins[k];
    CK(cudaEventRecord(b->ev_fork[0], b->stream));
    for (size_t i = 0; i < B.groups.size(); ++i) {
        CK(cudaStreamWaitEvent(b->side[i], b->ev_fork[0], 0));
        for (uint32_t s = 0; s < steps; ++s) chain_step(b, b->groups[B.groups[i]], b->side[i]);
        CK(cudaEventRecord(b->ev_join[i], b->side[i]));
    }
    for (size_t i = 0; i < B.groups.size(); ++i) CK(cudaStreamWaitEvent(b->stream, b->ev_join[i], 0));
    const cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) {
        set_error(std::string("batch kernel launch: ") + cudaGetErrorString(err));
        return FDTD_ERR_CUDA;
    }
    return FDTD_OK;
}

int bin_step(fdtd_batch_s* b, size_t k) {
    if (b->chains > 1) return bin_chains(b, k, 1);
    const fdtd_batch_s::Bin& B = b->bins[k];
    const size_t ng = B.groups.size();
    for (int gi : B.groups) launch_group_volt(b->groups[gi], b->d_jobs.p, b->XC, b->stages, b->stream, b->ty);
    for (int gi : B.groups) launch_group_curr(b->groups[gi], b->d_jobs.p, b->XC, b->stages, b->stream, b->ty);
    k_batch_energy_planes<<<dim3((unsigned)B.max_planes, (unsigned)B.count), 256, 0, b->stream>>>(b->d_adv.p + B.first);
    k_batch_advance<<<(unsigned)B.count, 256, 0, b->stream>>>(b->d_adv.p + B.first, kEps0, kMue0);
    b->last_launches += 2 * ng + 2;
    const cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) {
        set_error(std::string("batch kernel launch: ") + cudaGetErrorString(err));
        return FDTD_ERR_CUDA;
    }
    return FDTD_OK;
}

int batch_graph(fdtd_batch_s* b) {
    if (b->graph) return FDTD_OK;
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    int rc = FDTD_OK;
    const uint64_t saved = b->last_launches;
    for (size_t bi = 0; bi < b->bins.size() && rc == FDTD_OK; ++bi) {
        if (b->chains > 1) {
            rc = bin_chains(b, bi, b->graph_steps);
            continue;
        }
        for (uint32_t k = 0; k < b->graph_steps && rc == FDTD_OK; ++k) rc = bin_step(b, bi);
    }
    b->last_launches = saved;
    const cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (ce != cudaSuccess) {
        set_error(std::string("cudaStreamEndCapture (batch): ") + cudaGetErrorString(ce));
        return FDTD_ERR_CUDA;
    }
    const cudaError_t ie = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) {
        b->graph = nullptr;
        set_error(std::string("cudaGraphInstantiate (batch): ") + cudaGetErrorString(ie));
        return FDTD_ERR_CUDA;
    }
    return FDTD_OK;
}

int build_batch(const fdtd_engine_t* engines, uint32_t n, const fdtd_batch_opts* o, fdtd_batch_s* b) {
    if (n == 0) {
        set_error("fdtd_batch_create: no jobs");
        return FDTD_ERR_ARG;
    }
    b->device = engines[0] ? engines[0]->device : 0;
    b->XC = (o && o->x_chunk > 0) ? o->x_chunk : 0;  // 0: chosen below from the batch's size
    b->stages = (o && o->stages > 0) ? o->stages : 3;
    b->blocks_per_sm = (o && o->blocks_per_sm != 0) ? std::max(-1, o->blocks_per_sm) : 0;
    b->graph_steps = (o && o->graph_steps > 0) ? (uint32_t)o->graph_steps : 8;
    b->bin_bytes = (o && o->bin_mib > 0) ? (uint64_t)o->bin_mib << 20 : 0;
    b->chains = (o && o->chains > 1) ? std::min(o->chains, 64) : 1;
    b->ty = (o && o->tile_y == 4) ? 4 : BATCH_TY;
    if (o && o->tile_y != 0 && o->tile_y != 4 && o->tile_y != 8) {
        set_error("fdtd_batch_create: tile_y must be 4 or 8 (0 = 8)");
        return FDTD_ERR_ARG;
    }
    if (b->stages < 3 || b->stages > TMA_MAX_STAGES) {
        set_error("fdtd_batch_create: stages must be 3..8");
        return FDTD_ERR_ARG;
    }
    CK(cudaSetDevice(b->device));
    CK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    CK(cudaEventCreate(&b->ev0));
    CK(cudaEventCreate(&b->ev1));
    int rc;
    for (uint32_t j = 0; j < n; ++j) {
        fdtd_engine_s* e = engines[j];
        if (!e) {
            set_error("fdtd_batch_create: null engine");
            return FDTD_ERR_ARG;
        }
        if (e->device != b->device) {
            set_error("fdtd_batch_create: all jobs must live on one device");
            return FDTD_ERR_ARG;
        }
        if ((rc = batch_refusal(e))) return rc;
        for (uint32_t k = 0; k < j; ++k)
            if (engines[k] == e) {
                set_error("fdtd_batch_create: a job appears twice");
                return FDTD_ERR_ARG;
            }
        if ((rc = engine_start(e))) return rc;
        CK(cudaStreamSynchronize(e->stream));
    }
    // L2 bins: first fit by decreasing footprint (one bin when binning is off)
    std::vector<std::vector<fdtd_engine_s*>> binned;
    {
        std::vector<fdtd_engine_s*> byfoot(engines, engines + n);
        std::vector<uint64_t> load;
        if (b->bin_bytes)
            std::stable_sort(byfoot.begin(), byfoot.end(),
                             [](const fdtd_engine_s* a, const fdtd_engine_s* c) { return a->device_bytes > c->device_bytes; });
        else
            binned.emplace_back();
        for (fdtd_engine_s* e : byfoot) {
            if (!b->bin_bytes) {
                binned[0].push_back(e);
                continue;
            }
            size_t k = 0;
            while (k < binned.size() && load[k] + e->device_bytes > b->bin_bytes) ++k;
            if (k == binned.size()) {
                binned.emplace_back();
                load.push_back(0);
            }
            binned[k].push_back(e);
            load[k] += e->device_bytes;
        }
    }
    // jobs stored bin by bin and, within a bin, kernel variant by kernel
    // variant; each variant's job range is split into `chains` ranges of
    // about equal node count (one group each)
    size_t max_groups = 1;
    for (size_t bi = 0; bi < binned.size(); ++bi) {
        fdtd_batch_s::Bin B;
        B.first = (int)b->jobs.size();
        B.count = (int)binned[bi].size();
        auto key_of = [](const fdtd_engine_s* e) {
            return std::make_tuple((int)e->E.idx16, (int)e->H.idx16, (int)e->geo_on, e->feat_e * 8 + e->feat_h);
        };
        std::vector<fdtd_engine_s*> jobs = binned[bi];
        std::stable_sort(jobs.begin(), jobs.end(),
                         [&](const fdtd_engine_s* a, const fdtd_engine_s* c) { return key_of(a) < key_of(c); });
        for (size_t lo = 0; lo < jobs.size();) {
            size_t hi = lo;
            uint64_t nodes = 0;
            while (hi < jobs.size() && key_of(jobs[hi]) == key_of(jobs[lo])) {
                nodes += (uint64_t)jobs[hi]->N[0] * jobs[hi]->N[1] * jobs[hi]->N[2];
                ++hi;
            }
            const int parts = (int)std::min<size_t>((size_t)b->chains, hi - lo);
            uint64_t acc = 0;
            int part = -1;
            for (size_t q = lo; q < hi; ++q) {
                fdtd_engine_s* e = jobs[q];
                const uint64_t en = (uint64_t)e->N[0] * e->N[1] * e->N[2];
                // the part whose node share holds this job's midpoint
                const int want = std::min(parts - 1, (int)((acc + en / 2) * (uint64_t)parts / std::max<uint64_t>(1, nodes)));
                if (want != part || part < 0) {
                    Group G;
                    G.bin = (int)bi;
                    G.e16 = e->E.idx16;
                    G.h16 = e->H.idx16;
                    G.geo = e->geo_on;
                    G.feat = e->feat_e;
                    G.feat_h = e->feat_h;
                    G.first = (int)b->jobs.size();
                    b->groups.push_back(std::move(G));
                    B.groups.push_back((int)b->groups.size() - 1);
                    part = want;
                }
                Group& G = b->groups.back();
                const int j = (int)b->jobs.size();
                b->jobs.push_back(e);
                G.jobs.push_back(j);
                G.count++;
                G.max_planes = std::max(G.max_planes, (int)e->N[0] - 1);
                b->total_nodes += en;
                B.max_planes = std::max(B.max_planes, (int)e->N[0] - 1);
                acc += en;
            }
            lo = hi;
        }
        max_groups = std::max(max_groups, B.groups.size());
        b->bins.push_back(std::move(B));
    }
    if (b->chains > 1) {
        b->side.resize(max_groups, nullptr);
        b->ev_join.resize(max_groups, nullptr);
        b->ev_fork.resize(1, nullptr);
        for (cudaStream_t& s : b->side) CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        for (cudaEvent_t& e : b->ev_join) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&b->ev_fork[0], cudaEventDisableTiming));
    }
    // descriptors
    std::vector<TmaMaps> hmaps(n);  // the jobs' tensor maps for the batch's ty-row tiles
    for (uint32_t j = 0; j < n; ++j)
        if ((rc = engine_tma_maps(b->jobs[j], &hmaps[j], (uint32_t)b->ty))) return rc;
    if ((rc = b->d_maps.alloc(n, b->device_bytes)) || (rc = b->d_jobs.alloc(n, b->device_bytes)) ||
        (rc = b->d_adv.alloc(n, b->device_bytes)) || (rc = b->d_status.alloc(4 * (size_t)n, b->device_bytes)))
        return rc;
    b->h_status.assign(4 * (size_t)n, 0);
    std::vector<BatchJob> hj(n);
    std::vector<AdvJob> ha(n);
    for (uint32_t j = 0; j < n; ++j) {
        fdtd_engine_s* e = b->jobs[j];
        std::memset(&hj[j], 0, sizeof(BatchJob));
        hj[j].g = e->g;
        hj[j].ti = e->ti;
        hj[j].maps = b->d_maps.p + j;
        hj[j].interval = (int)e->interval;
        hj[j].energy = e->energy_on_probe ? 1 : 0;
        std::memset(&ha[j], 0, sizeof(AdvJob));
        ha[j].d_ts = e->p_ts();
        ha[j].ps = e->ps;
        ha[j].g = e->g;
        ha[j].interval = (int)e->interval;
        ha[j].energy_valid = e->energy_on_probe ? 1 : 0;
        ha[j].ctl = e->ctl.p;
        ha[j].out = b->d_status.p + 4 * (size_t)j;
        CK(cudaMemcpyAsync(b->d_status.p + 4 * (size_t)j, e->ctl.p, 4 * sizeof(int), cudaMemcpyDeviceToDevice,
                           b->stream));
    }
    CK(cudaMemcpyAsync(b->d_maps.p, hmaps.data(), n * sizeof(TmaMaps), cudaMemcpyHostToDevice, b->stream));
    CK(cudaMemcpyAsync(b->d_jobs.p, hj.data(), n * sizeof(BatchJob), cudaMemcpyHostToDevice, b->stream));
    CK(cudaMemcpyAsync(b->d_adv.p, ha.data(), n * sizeof(AdvJob), cudaMemcpyHostToDevice, b->stream));
    // work lists and persistent grid sizes
    int sms = 0;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device));
    if (b->XC == 0) {
        std::vector<const uint32_t*> lines;
        for (const fdtd_engine_s* e : b->jobs) lines.push_back(e->N);
        b->XC = auto_x_chunk(lines, (uint64_t)(1024 / (32 * b->ty)) * (uint64_t)sms, b->ty);
    }
    const size_t maxsm = std::max(stage_smem(false, true, true, b->stages, 8), stage_smem(false, true, true, b->stages, 4));
    if (maxsm > 48 * 1024 && (rc = batch_smem_attrs((int)maxsm))) return rc;
    for (Group& G : b->groups) {
        std::vector<WorkItem> wE, wH;
        for (int j : G.jobs) {
            const fdtd_engine_s* e = b->jobs[j];
            const int bxE = (e->ti.ne[2] + 31) / 32, byE = (e->ti.ne[1] + b->ty - 1) / b->ty,
                      bzE = (e->ti.ne[0] + b->XC - 1) / b->XC;
            for (int z = 0; z < bzE; ++z)
                for (int y = 0; y < byE; ++y)
                    for (int x = 0; x < bxE; ++x) wE.push_back(WorkItem{j, x, y, z});
            const int bxH = ((int)e->N[2] - 1 + 31) / 32, byH = ((int)e->N[1] - 1 + b->ty - 1) / b->ty,
                      bzH = ((int)e->N[0] - 1 + b->XC - 1) / b->XC;
            for (int z = 0; z < bzH; ++z)
                for (int y = 0; y < byH; ++y)
                    for (int x = 0; x < bxH; ++x) wH.push_back(WorkItem{j, x, y, z});
        }
        G.nE = (int)wE.size();
        G.nH = (int)wH.size();
        if ((rc = G.itE.alloc(wE.size(), b->device_bytes)) || (rc = G.itH.alloc(wH.size(), b->device_bytes))) return rc;
        CK(cudaMemcpyAsync(G.itE.p, wE.data(), wE.size() * sizeof(WorkItem), cudaMemcpyHostToDevice, b->stream));
        CK(cudaMemcpyAsync(G.itH.p, wH.data(), wH.size() * sizeof(WorkItem), cudaMemcpyHostToDevice, b->stream));
        const bool up = (G.feat & FEAT_UPML) != 0;
        G.smemE = stage_smem(G.e16, up, (G.feat & FEAT_ADE) != 0, b->stages, b->ty);
        G.smemH = stage_smem(G.h16, up, false, b->stages, b->ty);
        int oE = occupancy(G, true, G.smemE, b->ty), oH = occupancy(G, false, G.smemH, b->ty);
        if (b->blocks_per_sm > 0) {
            oE = std::min(oE, b->blocks_per_sm);
            oH = std::min(oH, b->blocks_per_sm);
        }
        G.gridE = std::max(1, std::min(G.nE, std::max(1, oE) * sms));
        G.gridH = std::max(1, std::min(G.nH, std::max(1, oH) * sms));
        if (b->blocks_per_sm < 0) {  // one block per work item: the hardware schedules the items
            G.gridE = std::max(1, G.nE);
            G.gridH = std::max(1, G.nH);
        }
    }
    CK(cudaStreamSynchronize(b->stream));
    return FDTD_OK;
}

}  // namespace
}  // namespace wipems

extern "C" {

int fdtd_batch_create(const fdtd_engine_t* engines, uint32_t n, const fdtd_batch_opts* opts, fdtd_batch_t* out) {
    if (!engines || !out) {
        set_error("fdtd_batch_create: null argument");
        return FDTD_ERR_ARG;
    }
    fdtd_batch_s* b = new (std::nothrow) fdtd_batch_s();
    if (!b) return FDTD_ERR_NOMEM;
    int rc;
    try {
        rc = build_batch(engines, n, opts, b);
    } catch (const std::bad_alloc&) {
        set_error("fdtd_batch_create: host allocation failed");
        rc = FDTD_ERR_NOMEM;
    }
    if (rc) {
        delete b;
        return rc;
    }
    *out = b;
    return FDTD_OK;
}

int fdtd_batch_accepts(fdtd_engine_t e, int* ok) {
    if (!e || !ok) return FDTD_ERR_ARG;
    const std::string keep = last_error();  // a query leaves the thread's last message alone
    *ok = batch_refusal(e) == FDTD_OK ? 1 : 0;
    set_error(keep);
    return FDTD_OK;
}

int fdtd_batch_destroy(fdtd_batch_t b) {
    if (!b) return FDTD_OK;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    delete b;
    return FDTD_OK;
}

int fdtd_batch_iterate(fdtd_batch_t b, uint32_t n) {
    if (!b) return FDTD_ERR_ARG;
    if (n == 0) return FDTD_OK;
    CK(cudaSetDevice(b->device));
    b->last_launches = 0;
    int rc;
    if (b->graph_steps > 1 && n >= b->graph_steps && (rc = batch_graph(b))) return rc;
    CK(cudaEventRecord(b->ev0, b->stream));
    uint32_t left = n;
    while (left > 0) {
        if (b->graph && left >= b->graph_steps) {
            CK(cudaGraphLaunch(b->graph, b->stream));
            b->last_launches += (b->chains > 1 ? 4 * b->groups.size() : 2 * b->groups.size() + 2 * b->bins.size()) *
                                b->graph_steps;
            left -= b->graph_steps;
            continue;
        }
        for (size_t bi = 0; bi < b->bins.size(); ++bi)
            if ((rc = bin_step(b, bi))) return rc;
        left -= 1;
    }
    CK(cudaEventRecord(b->ev1, b->stream));
    CK(cudaEventSynchronize(b->ev1));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
    b->last_ms = ms;
    // every job's control words in one copy: numTS, done, error word
    const size_t nj = b->jobs.size();
    CK(cudaMemcpyAsync(b->h_status.data(), b->d_status.p, nj * 4 * sizeof(int), cudaMemcpyDeviceToHost, b->stream));
    CK(cudaStreamSynchronize(b->stream));
    int first_rc = FDTD_OK;
    for (size_t j = 0; j < nj; ++j) {
        fdtd_engine_s* e = b->jobs[j];
        const int* c = &b->h_status[4 * j];
        e->ts = (uint32_t)c[0];
        e->done = c[3] != 0;
        if (c[2] && first_rc == FDTD_OK) first_rc = engine_decode_error(c[2]);
    }
    return first_rc;
}

int fdtd_batch_info(fdtd_batch_t b, fdtd_batch_stats* st) {
    if (!b || !st) return FDTD_ERR_ARG;
    std::memset(st, 0, sizeof(*st));
    st->num_jobs = (uint32_t)b->jobs.size();
    st->num_groups = (uint32_t)b->groups.size();
    st->num_bins = (uint32_t)b->bins.size();
    st->total_nodes = b->total_nodes;
    for (const Group& G : b->groups) {
        st->work_items += (uint64_t)G.nE + G.nH;
        st->persistent_blocks = std::max<uint32_t>(st->persistent_blocks, (uint32_t)std::max(G.gridE, G.gridH));
    }
    st->device_bytes = b->device_bytes;
    st->last_ms = b->last_ms;
    st->last_launches = b->last_launches;
    st->x_chunk = (uint32_t)b->XC;
    return FDTD_OK;
}

}  // extern "C"
