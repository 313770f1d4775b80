// mz_sort_keys_noalloc: the stable counting sort of sort_particles! reduced to
// its permutation, for callers that cannot allocate device memory.
//
// Some host programs may not call cudaMalloc / cudaFree at all once they are
// running: a process whose device memory is already owned by another
// framework's caching allocator (a Julia or PyTorch pool that reserved the
// GPU), or a latency-critical loop that must not take the implicit device-wide
// synchronisation an allocation or free performs.  The regular entry points
// keep their per-cell counters in memory the library allocates with the
// domain; this entry point keeps them instead in one file-scope
// `static __device__` array, sized for MZ_NOALLOC_MAX_CELLS cells, that every
// GPU loading the library holds until the process exits.
//
// The caller passes the keys, the permutation output and the cell-start
// output, all in device memory, and the stream.  The scratch array is shared
// by every call: each call clears what must start at zero, and calls that
// overlap on the GPU (different streams or devices sharing it concurrently on
// one device) race on it -- serialise them.  Before returning, a call waits
// for its stream (a wait on that stream alone, not the device-wide
// synchronisation an allocation or free can take) to read the word that
// reports keys outside [0, n_cells).
#include "mz_host.h"
#include "sortnet.cuh"

#include <cuda.h>

#include <cstdio>
#include <mutex>

using namespace mz;

namespace {

constexpr int kMaxDevices = 64;

// [0, MAX): per-cell counts, [MAX, 2 MAX): per-cell cursors, [2 MAX]: status
static __device__ __align__(256) int32_t g_noalloc_scratch[2 * MZ_NOALLOC_MAX_CELLS + 64];

std::mutex g_mutex;
// the array's device address per device, and the id of the CUDA context it
// belongs to: a device's primary context that was reset (cudaDeviceReset) is
// recreated with a new id and the array with a new address
struct ScratchAddr {
    unsigned long long ctx_id;
    int32_t* addr;
};
ScratchAddr g_scratch[kMaxDevices] = {};

// unique id of the calling thread's current CUDA context (cuCtxGetId, taken
// from the driver through the runtime so the library needs no libcuda link);
// 0 when there is none or the driver cannot say
unsigned long long current_context_id()
{
    using GetCurrent = CUresult (*)(CUcontext*);
    using GetId = CUresult (*)(CUcontext, unsigned long long*);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    static bool looked_up = false;
    if (!looked_up) {
        looked_up = true;
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<GetCurrent>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<GetId>(f);
        cudaGetLastError();
    }
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (get_current && get_id && get_current(&ctx) == CUDA_SUCCESS && ctx && get_id(ctx, &id) == CUDA_SUCCESS)
        return id;
    return 0;
}

__device__ __forceinline__ int32_t clamp_key(int32_t k, int32_t n_cells, int32_t* status)
{
    if (k < 0 || k >= n_cells) {
        atomicOr(status, 1);
        k = k < 0 ? 0 : n_cells - 1;
    }
    return k;
}

__global__ void k_na_clear(int32_t* scratch, int32_t n_cells)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_cells; i += gridDim.x * blockDim.x) {
        scratch[i] = 0;
        scratch[MZ_NOALLOC_MAX_CELLS + i] = 0;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) scratch[2 * MZ_NOALLOC_MAX_CELLS] = 0;
}

__global__ void k_na_count(const int32_t* keys, int64_t n, int32_t n_cells, int32_t* scratch)
{
    const int lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x + threadIdx.x - lane; base < n; base += stride) {
        const int64_t i = base + lane;
        const bool in = i < n;
        const unsigned m = __ballot_sync(0xFFFFFFFFu, in);
        if (!in) continue;
        const int32_t k = clamp_key(keys[i], n_cells, scratch + 2 * MZ_NOALLOC_MAX_CELLS);
        warp_agg_add(scratch, k, m);
    }
}

// exclusive scan of the counts into the caller's cell_start[0 .. n_cells]
__global__ void __launch_bounds__(1024) k_na_scan(const int32_t* scratch, int32_t n, int32_t* cell_start)
{
    __shared__ long long warp_tot[32];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const int chunk = (n + blockDim.x - 1) / blockDim.x;
    const int c0 = min(n, t * chunk), c1 = min(n, c0 + chunk);
    long long local = 0;
    for (int c = c0; c < c1; ++c) local += scratch[c];
    long long incl = local;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const long long v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= o) incl += v;
    }
    if (lane == 31) warp_tot[w] = incl;
    __syncthreads();
    if (w == 0) {
        const long long v = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0;
        long long vi = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long u = __shfl_up_sync(0xFFFFFFFFu, vi, o);
            if (lane >= o) vi += u;
        }
        warp_tot[lane] = vi - v;
        if (lane == 31) cell_start[n] = (int32_t)vi;
    }
    __syncthreads();
    long long run = warp_tot[w] + (incl - local);
    for (int c = c0; c < c1; ++c) {
        cell_start[c] = (int32_t)run;
        run += scratch[c];
    }
}

__global__ void k_na_scatter(const int32_t* keys, int64_t n, int32_t n_cells, const int32_t* cell_start,
                             int32_t* scratch, int32_t* perm)
{
    const int lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x + threadIdx.x - lane; base < n; base += stride) {
        const int64_t i = base + lane;
        const bool in = i < n;
        const unsigned m = __ballot_sync(0xFFFFFFFFu, in);
        if (!in) continue;
        const int32_t k = clamp_key(keys[i], n_cells, scratch + 2 * MZ_NOALLOC_MAX_CELLS);
        const int32_t pos = cell_start[k] + warp_agg_ticket(scratch + MZ_NOALLOC_MAX_CELLS, k, m);
        perm[pos] = (int32_t)i;
    }
}

template <int E>
__device__ __forceinline__ void sort_in_place_regs(int32_t* seg, int32_t N)
{
    const int lane = threadIdx.x & 31;
    int32_t v[E];
#pragma unroll
    for (int r = 0; r < E; ++r) {
        const int q = r * 32 + lane;
        v[r] = q < N ? seg[q] : INT_MAX;
    }
    warp_bitonic<E>(v);
#pragma unroll
    for (int r = 0; r < E; ++r) {
        const int q = r * 32 + lane;
        if (q < N) seg[q] = v[r];
    }
}

// tickets arrive in any order; sorting each cell's segment restores the
// stable order (grid_sorting.jl:101-106)
__global__ void __launch_bounds__(256) k_na_segments(int32_t n_cells, const int32_t* cell_start, int32_t* perm)
{
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < n_cells; c += warps) {
        const int32_t s = cell_start[c], N = cell_start[c + 1] - s;
        int32_t* seg = perm + s;
        if (N <= 1) continue;
        if (N <= 32) sort_in_place_regs<1>(seg, N);
        else if (N <= 64) sort_in_place_regs<2>(seg, N);
        else if (N <= 128) sort_in_place_regs<4>(seg, N);
        else if (N <= 256) sort_in_place_regs<8>(seg, N);
        else if (N <= 512) sort_in_place_regs<16>(seg, N);
        else if (N <= 1024) sort_in_place_regs<32>(seg, N);
        else warp_oddeven_sort(seg, N);
    }
}

// device address of the scratch array for the current device: looked up
// (cudaGetSymbolAddress, with the device current) on the first call in each
// CUDA context of the device, then taken from the cache
int32_t* scratch_for_current_device(int* device_out)
{
    int dev = 0;
    MZ_CK(cudaGetDevice(&dev));
    MZ_REQUIRE(dev >= 0 && dev < kMaxDevices, "mz_sort_keys_noalloc: device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_mutex);
    *device_out = dev;
    const unsigned long long id = current_context_id();
    if (id != 0 && g_scratch[dev].ctx_id == id && g_scratch[dev].addr) return g_scratch[dev].addr;
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess)
        throw MzError(MZ_E_CUDA, std::string("mz_sort_keys_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    // the lookup made the device's context current on this thread; without a
    // context id (an old driver) the address is looked up on every call
    g_scratch[dev].ctx_id = current_context_id();
    g_scratch[dev].addr = static_cast<int32_t*>(p);
    return g_scratch[dev].addr;
}

}  // namespace

extern "C" {

int mz_sort_keys_noalloc(void* stream, const int32_t* d_keys, int64_t n, int32_t n_cells, int32_t* d_perm,
                         int32_t* d_cell_start)
{
    try {
        MZ_REQUIRE(n >= 0 && n < (1ll << 31) - 1, "mz_sort_keys_noalloc: n must be in [0, 2^31 - 1)");
        MZ_REQUIRE(n_cells >= 1 && n_cells <= MZ_NOALLOC_MAX_CELLS,
                   "mz_sort_keys_noalloc: n_cells must be in [1, MZ_NOALLOC_MAX_CELLS]");
        MZ_REQUIRE(d_cell_start && (n == 0 || (d_keys && d_perm)), "mz_sort_keys_noalloc: NULL device pointer");
        int dev = 0;
        int32_t* scratch = scratch_for_current_device(&dev);
        int sms = 0;
        MZ_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        cudaStream_t st = (cudaStream_t)stream;
        const int cblocks = (int)std::max<int64_t>(1, std::min<int64_t>(div_up(n_cells, 256), (int64_t)sms * 4));
        k_na_clear<<<cblocks, 256, 0, st>>>(scratch, n_cells);
        MZ_CK(cudaGetLastError());
        const int pblocks = (int)std::max<int64_t>(1, std::min<int64_t>(div_up(n, 256), (int64_t)sms * 8));
        if (n > 0) {
            k_na_count<<<pblocks, 256, 0, st>>>(d_keys, n, n_cells, scratch);
            MZ_CK(cudaGetLastError());
        }
        k_na_scan<<<1, 1024, 0, st>>>(scratch, n_cells, d_cell_start);
        MZ_CK(cudaGetLastError());
        if (n > 0) {
            k_na_scatter<<<pblocks, 256, 0, st>>>(d_keys, n, n_cells, d_cell_start, scratch, d_perm);
            MZ_CK(cudaGetLastError());
            const int sblocks = (int)std::max<int64_t>(1, std::min<int64_t>(div_up((int64_t)n_cells * 32, 256),
                                                                            (int64_t)sms * 16));
            k_na_segments<<<sblocks, 256, 0, st>>>(n_cells, d_cell_start, d_perm);
            MZ_CK(cudaGetLastError());
        }
        int32_t status = 0;
        MZ_CK(cudaMemcpyAsync(&status, scratch + 2 * MZ_NOALLOC_MAX_CELLS, sizeof status, cudaMemcpyDeviceToHost, st));
        MZ_CK(cudaStreamSynchronize(st));
        if (status) throw MzError(MZ_E_STATE, "mz_sort_keys_noalloc: key outside [0, n_cells) (clamped)");
    } catch (MzError& e) {
        fprintf(stderr, "merzgpu: %s\n", e.what());
        return e.code;
    } catch (std::exception& e) {
        fprintf(stderr, "merzgpu: %s\n", e.what());
        return MZ_E_ARG;
    }
    return MZ_OK;
}

}  // extern "C"
