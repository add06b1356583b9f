// Allocation-free macroscopic moments of a Shakhov state (g, h).
//
// Who this is for: callers that cannot call cudaMalloc.  A host framework
// that owns all device memory in its own pool hands an operator nothing but
// its input and output buffers; a serving or real-time loop with a fixed
// memory budget must not call cudaMalloc / cudaFree (which synchronize the
// device) between steps.  Creating a meso_ctx allocates its tables and
// scratch on the device, so those callers get this one entry point instead:
// every buffer it reads or writes is the caller's, and its only scratch is
// the file-scope device array below, reserved once when the library's device
// code is loaded on a GPU and held there until the process exits.
//
// Work split: each cell's velocities are cut into ngroup contiguous groups;
// one warp sums one (cell, group) and writes 8 partial sums to the scratch
// array; the last block of a cell block to finish (a counter per cell block,
// also in the scratch array) adds the groups' partials in group order and
// writes rho, u, T, q.  The sums are those of initial() with the equilibrium
// recomputed as moments (cdugks_shakhov.cpp:102-169), evaluated in the same
// expressions; only the order of the velocity sums differs.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "meso_gpu.h"

namespace meso_host {
int fail(int code, const std::string &msg);
}

namespace {

constexpr int kCellsPerBlock = 8;  // one warp per cell
constexpr int kThreads = kCellsPerBlock * 32;
constexpr int kMaxCells = MESO_NOALLOC_MAX_CELLS;
constexpr int kMaxCellBlocks = kMaxCells / kCellsPerBlock;
constexpr size_t kCounterBytes = sizeof(unsigned) * kMaxCellBlocks;       // 64 KiB
constexpr size_t kPartialDoubles = (size_t)kMaxCells * 8;                  // ngroup * ncell * 8 <= this
constexpr size_t kScratchBytes = kCounterBytes + sizeof(double) * kPartialDoubles;  // 8 MiB + 64 KiB
static_assert(kMaxCells % kCellsPerBlock == 0, "cell blocks must tile the maximum");
static_assert(kCounterBytes % 256 == 0, "partials start on a 256-byte boundary");

// The scratch array.  In host code this name is only a handle for
// cudaGetSymbolAddress, never a device address.
static __device__ __align__(256) unsigned char g_moments_scratch[kScratchBytes];

template <int DIM>
__device__ __forceinline__ double dot3(double ax, double ay, double az, double bx, double by, double bz) {
    if (DIM == 2) return ax * bx + ay * by;
    return ax * bx + ay * by + az * bz;
}

template <int DIM>
__global__ void __launch_bounds__(kThreads) k_moments_split(const double *__restrict__ g, const double *__restrict__ h,
                                                            int C, int NV, const double *__restrict__ xi,
                                                            const double *__restrict__ w,
                                                            const double *__restrict__ u0, double Cv, int ngroup,
                                                            unsigned char *scratch, double *rho_c, double *u_c,
                                                            double *T_c, double *q_c) {
    unsigned *count = reinterpret_cast<unsigned *>(scratch);
    double *part = reinterpret_cast<double *>(scratch + kCounterBytes);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int c = blockIdx.x * kCellsPerBlock + warp;
    const int grp = blockIdx.y;
    const int per = (NV + ngroup - 1) / ngroup;
    const int p0 = grp * per, p1 = min(NV, p0 + per);
    double v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (c < C) {
        const double ux = u0[3 * c], uy = u0[3 * c + 1], uz = u0[3 * c + 2];
        const size_t base = (size_t)c * NV;
        for (int p = p0 + lane; p < p1; p += 32) {
            const double x = xi[3 * p], y = xi[3 * p + 1], z = xi[3 * p + 2];
            const double cx = x - ux, cy = y - uy, cz = z - uz;
            const double cc = dot3<DIM>(cx, cy, cz, cx, cy, cz);
            const double gv = g[base + p], hv = h[base + p];
            const double wp = w[p];
            const double kk = dot3<DIM>(x, y, z, x, y, z);
            v[0] += wp * gv;
            const double wg = wp * gv;
            v[1] += x * wg;
            v[2] += y * wg;
            v[3] += z * wg;
            v[4] += wp * (kk * gv + hv);
            const double s = cc * gv + hv;
            v[5] += (cx * wp) * s;
            v[6] += (cy * wp) * s;
            v[7] += (cz * wp) * s;
        }
    }
#pragma unroll
    for (int k = 0; k < 8; ++k)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
    if (c < C && lane < 8) {
        double mine = v[0];
#pragma unroll
        for (int k = 1; k < 8; ++k)
            if (lane == k) mine = v[k];
        part[((size_t)grp * C + c) * 8 + lane] = mine;
    }
    // last-block-done: partials visible device-wide before the counter moves
    __threadfence();
    __syncthreads();
    __shared__ int is_last;
    if (threadIdx.x == 0) is_last = atomicAdd(&count[blockIdx.x], 1u) == (unsigned)(ngroup - 1);
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    if (c >= C) return;
    double s = 0.0;
    if (lane < 8)
        for (int q = 0; q < ngroup; ++q) s += __ldcg(&part[((size_t)q * C + c) * 8 + lane]);
    double t[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) t[k] = __shfl_sync(0xffffffffu, s, k);
    if (lane != 0) return;
    const double rho = t[0];
    const double rhoE = 0.5 * t[4];
    const double r = 1.0 / rho;
    const double ux = t[1] * r, uy = t[2] * r, uz = t[3] * r;
    const double T = (rhoE / rho - dot3<DIM>(ux * 0.5, uy * 0.5, uz * 0.5, ux, uy, uz)) / Cv;
    rho_c[c] = rho;
    u_c[3 * c] = ux;
    u_c[3 * c + 1] = uy;
    u_c[3 * c + 2] = uz;
    T_c[c] = T;
    q_c[3 * c] = t[5] * 0.5;
    q_c[3 * c + 1] = t[6] * 0.5;
    q_c[3 * c + 2] = t[7] * 0.5;
}

// Per-device set-up: the scratch array's device address and the SM count.
constexpr int kMaxDevices = 64;
struct DeviceSlot {
    void *scratch = nullptr;
    int sms = 0;
};
std::mutex g_setup_mu;
DeviceSlot g_slots[kMaxDevices];

int device_setup(DeviceSlot &out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return meso_host::fail(MESO_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return meso_host::fail(MESO_ERR_CUDA, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_setup_mu);
    DeviceSlot &s = g_slots[dev];
    if (!s.scratch) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_moments_scratch);
        if (e != cudaSuccess || !p)
            return meso_host::fail(MESO_ERR_CUDA,
                                   std::string("cudaGetSymbolAddress(moments scratch): ") + cudaGetErrorString(e));
        int sms = 0;
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess || sms <= 0)
            return meso_host::fail(MESO_ERR_CUDA, std::string("SM count: ") + cudaGetErrorString(e));
        s.sms = sms;
        s.scratch = p;
    }
    out = s;
    return MESO_OK;
}

// Where a caller's pointer lives.  0: device (or managed) memory of device `dev`; 1: anything else
// (pageable or page-locked host memory, another GPU's memory, an unknown address).  An error that
// the attribute query itself raises is this call's own (the entry point refuses to run while an
// earlier error is pending), so it is cleared here.
int where(const void *p, int dev) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    if (a.type == cudaMemoryTypeManaged) return 0;
    return a.type == cudaMemoryTypeDevice && a.device == dev ? 0 : 1;
}

}  // namespace

extern "C" int meso_shakhov_moments_noalloc(const double *g, const double *h, int32_t ncell, int32_t nv, int32_t dim,
                                            const double *xi, const double *w, const double *u0, double R, double K,
                                            double *rho, double *u, double *T, double *q, void *stream) {
    if (ncell <= 0 || nv <= 0) return meso_host::fail(MESO_ERR_INVALID, "ncell and nv must be positive");
    if (ncell > kMaxCells)
        return meso_host::fail(MESO_ERR_CAPACITY, "meso_shakhov_moments_noalloc: ncell = " + std::to_string(ncell) +
                                                      " exceeds MESO_NOALLOC_MAX_CELLS = " + std::to_string(kMaxCells));
    if (dim != 2 && dim != 3) return meso_host::fail(MESO_ERR_INVALID, "dim must be 2 or 3");
    if (!(R > 0.0) || !(K >= 0.0)) return meso_host::fail(MESO_ERR_INVALID, "R must be > 0 and K >= 0");
    // An error left pending by earlier CUDA work of the caller stays theirs to read: it is neither
    // cleared here nor reported as this call's launch failure.
    const cudaError_t pending = cudaPeekAtLastError();
    if (pending == cudaErrorNoDevice || pending == cudaErrorInsufficientDriver)  // no GPU to hold the arrays
        return meso_host::fail(MESO_ERR_INVALID, std::string("no usable CUDA device (") + cudaGetErrorString(pending) +
                                                     "): the arrays cannot be device memory of the current GPU");
    if (pending != cudaSuccess)
        return meso_host::fail(MESO_ERR_CUDA, std::string("a CUDA error is pending from before this call: ") +
                                                  cudaGetErrorString(pending));
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        dev = -1;
    }
    const void *ptrs[] = {g, h, xi, w, u0, rho, u, T, q};
    for (const void *p : ptrs)
        if (!p || where(p, dev) != 0)
            return meso_host::fail(MESO_ERR_INVALID,
                                   "every array must be device (or managed) memory of the current GPU");
    DeviceSlot slot;
    int rc = device_setup(slot);
    if (rc) return rc;
    const cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int ncb = (ncell + kCellsPerBlock - 1) / kCellsPerBlock;
    // about two waves of 8 resident blocks per SM, groups of at least 32 velocities, partials within the array
    const int target = 2 * 8 * slot.sms;
    int ngroup = (target + ncb - 1) / ncb;
    ngroup = ngroup < (nv + 31) / 32 ? ngroup : (nv + 31) / 32;
    const int fit = (int)(kPartialDoubles / ((size_t)ncell * 8));
    ngroup = ngroup < fit ? ngroup : fit;
    ngroup = ngroup < 65535 ? ngroup : 65535;
    ngroup = ngroup > 1 ? ngroup : 1;
    // no empty group: with per = ceil(nv / ngroup) velocities each, ceil(nv / per) groups cover nv
    {
        const int per = (nv + ngroup - 1) / ngroup;
        ngroup = (nv + per - 1) / per;
    }
    // the counters must start at zero; the partials need no clearing (each is written before it is read)
    cudaError_t e = cudaMemsetAsync(slot.scratch, 0, sizeof(unsigned) * (size_t)ncb, st);
    if (e != cudaSuccess) return meso_host::fail(MESO_ERR_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
    const double Cv = (K + 3.0) * R * 0.5;
    const dim3 grid(ncb, ngroup);
    unsigned char *scr = static_cast<unsigned char *>(slot.scratch);
    if (dim == 2)
        k_moments_split<2><<<grid, kThreads, 0, st>>>(g, h, ncell, nv, xi, w, u0, Cv, ngroup, scr, rho, u, T, q);
    else
        k_moments_split<3><<<grid, kThreads, 0, st>>>(g, h, ncell, nv, xi, w, u0, Cv, ngroup, scr, rho, u, T, q);
    e = cudaGetLastError();
    if (e != cudaSuccess) return meso_host::fail(MESO_ERR_CUDA, std::string("moments launch: ") + cudaGetErrorString(e));
    return MESO_OK;
}
