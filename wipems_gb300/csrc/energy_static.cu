// Field energy without any device allocation.
//
// fdtd_engine_energy reduces the engine's fields into a small accumulator
// buffer the engine allocated with cudaMalloc.  Callers that own their field
// arrays but may not allocate device memory -- code running inside a
// pre-sized memory budget, a real-time loop that must not touch the
// allocator, or an embedding application whose allocator is off limits --
// use fdtd_field_energy_static instead: the per-plane partial sums live in
// the file-scope array below, which every GPU that loads this library holds
// until the process exits.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>

#include "fdtd_host.h"

namespace wipems {
namespace {

// one (sum V^2, sum I^2) pair per x-plane of the energy domain
constexpr uint32_t kStaticMaxPlanes = 4096;
static __device__ __align__(256) double g_energy_scratch[2 * kStaticMaxPlanes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
double* g_scratch_ptr[kMaxDevices] = {nullptr};

// Block p sums V^2 and I^2 over plane x = p (y < Ny-1, z < Nz-1), as
// Engine_Interface_FDTD::CalcFastEnergy (engine_interface_fdtd.cpp:292-337)
// does over the whole grid, and writes the pair to scratch[2p].
__global__ void k_plane_energy(const float* __restrict__ V, const float* __restrict__ I, uint32_t Ny, uint32_t Nz,
                               uint32_t pitch, uint64_t comp, double* scratch) {
    const uint32_t x = blockIdx.x;
    double es = 0.0, hs = 0.0;
    const uint64_t plane = (uint64_t)x * Ny * pitch;
    const uint32_t cnt = (Ny - 1) * (Nz - 1);
    for (uint32_t i = threadIdx.x; i < cnt; i += blockDim.x) {
        const uint32_t y = i / (Nz - 1), z = i - y * (Nz - 1);
        const uint64_t o = plane + (uint64_t)y * pitch + z;
#pragma unroll
        for (int n = 0; n < 3; ++n) {
            const float v = V[n * comp + o];
            const float c = I[n * comp + o];
            es += (double)__fmul_rn(v, v);
            hs += (double)__fmul_rn(c, c);
        }
    }
    __shared__ double se[32], sh[32];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        es += __shfl_down_sync(0xffffffffu, es, off);
        hs += __shfl_down_sync(0xffffffffu, hs, off);
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) {
        se[w] = es;
        sh[w] = hs;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
            a += se[k];
            b += sh[k];
        }
        scratch[2 * x] = a;
        scratch[2 * x + 1] = b;
    }
}

// Sums the plane pairs in plane order and writes eps0*E + mu0*H.
__global__ void k_planes_total(const double* scratch, uint32_t planes, double eps0, double mue0, double* out) {
    if (threadIdx.x != 0) return;
    double a = 0.0, b = 0.0;
    for (uint32_t p = 0; p < planes; ++p) {
        a += scratch[2 * p];
        b += scratch[2 * p + 1];
    }
    out[0] = eps0 * a + mue0 * b;
}

// Device address of the static scratch array on the current device, looked
// up once per device, on the first call made with that device current
// (cudaGetSymbolAddress; no allocation).  The cached address belongs to
// the device's context: after cudaDeviceReset the library's module is
// loaded anew and the cached address is stale, so this entry point must not
// be called again in a process that reset the device.
int scratch_address(int dev, double** out) {
    if (dev < 0 || dev >= kMaxDevices) {
        set_error("fdtd_field_energy_static: device ordinal out of range");
        return FDTD_ERR_ARG;
    }
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_energy_scratch);
        if (e != cudaSuccess || !p) {
            set_error(std::string("fdtd_field_energy_static: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
            return FDTD_ERR_CUDA;
        }
        g_scratch_ptr[dev] = static_cast<double*>(p);
    }
    *out = g_scratch_ptr[dev];
    return FDTD_OK;
}

}  // namespace
}  // namespace wipems

using namespace wipems;

extern "C" int fdtd_field_energy_static(const float* volt, const float* curr, const uint32_t num_lines[3],
                                        uint32_t z_pitch, void* stream, double* energy) {
    if (!volt || !curr || !num_lines || !energy) {
        set_error("fdtd_field_energy_static: null argument");
        return FDTD_ERR_ARG;
    }
    const uint32_t Nx = num_lines[0], Ny = num_lines[1], Nz = num_lines[2];
    if (Nx < 2 || Ny < 2 || Nz < 2 || z_pitch < Nz) {
        set_error("fdtd_field_energy_static: need >= 2 lines per axis and z_pitch >= num_lines[2]");
        return FDTD_ERR_ARG;
    }
    if (Nx - 1 > kStaticMaxPlanes) {
        set_error("fdtd_field_energy_static: num_lines[0]-1 = " + std::to_string(Nx - 1) +
                  " planes exceeds the static scratch capacity of " + std::to_string(kStaticMaxPlanes));
        return FDTD_ERR_ARG;
    }
    int dev = 0;
    cudaError_t ce = cudaGetDevice(&dev);
    if (ce != cudaSuccess) {
        set_error(std::string("fdtd_field_energy_static: cudaGetDevice: ") + cudaGetErrorString(ce));
        return FDTD_ERR_CUDA;
    }
    double* scratch = nullptr;
    int rc = scratch_address(dev, &scratch);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const uint64_t comp = (uint64_t)Nx * Ny * z_pitch;
    k_plane_energy<<<Nx - 1, 256, 0, s>>>(volt, curr, Ny, Nz, z_pitch, comp, scratch);
    k_planes_total<<<1, 32, 0, s>>>(scratch, Nx - 1, kEps0, kMue0, energy);
    ce = cudaGetLastError();
    if (ce != cudaSuccess) {
        set_error(std::string("fdtd_field_energy_static: kernel launch: ") + cudaGetErrorString(ce));
        return FDTD_ERR_CUDA;
    }
    return FDTD_OK;
}
