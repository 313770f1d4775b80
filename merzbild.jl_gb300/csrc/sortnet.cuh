// Per-cell segment sort + gather used by the counting sort (sort.cu) and the
// fused step (step.cu).  The scatter pass hands out slots inside a cell's
// segment in arbitrary (atomic) order; sorting the segment's source slots
// ascending restores the stable order of sort_particles!
// (grid_sorting.jl:101-106), after which the particle columns are gathered.
#pragma once

#include <climits>

#include "mz_internal.cuh"

namespace mz {

// Ascending bitonic sort of 32*E keys held register-major (position r*32+lane).
template <int E>
__device__ __forceinline__ void warp_bitonic(int32_t (&v)[E])
{
    const int lane = threadIdx.x & 31;
    constexpr int P = 32 * E;
#pragma unroll
    for (int k = 2; k <= P; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
            if (j >= 32) {
                const int jr = j >> 5;
#pragma unroll
                for (int r = 0; r < E; ++r) {
                    const int rp = r ^ jr;
                    if (rp > r) {
                        const bool asc = ((r * 32) & k) == 0;
                        const int32_t a = v[r], b = v[rp];
                        const bool sw = asc ? (a > b) : (a < b);
                        v[r] = sw ? b : a;
                        v[rp] = sw ? a : b;
                    }
                }
            } else {
#pragma unroll
                for (int r = 0; r < E; ++r) {
                    const int p = r * 32 + lane;
                    const int32_t o = __shfl_xor_sync(0xFFFFFFFFu, v[r], j);
                    const bool lower = (lane & j) == 0;
                    const bool asc = (p & k) == 0;
                    v[r] = (lower == asc) ? min(v[r], o) : max(v[r], o);
                }
            }
        }
    }
}

// The same network with its (k, j) stages in runtime loops: fully unrolled,
// the 32- and 64-row sorts are more code than the instruction caches hold
// (instruction fetch was the first stall of the gathers that run them).  A
// stage within a row is one unrolled pass of shuffles; a stage across rows
// (j >= 32) dispatches on the row distance to an unrolled pass.
template <int JR, int E>
__device__ __forceinline__ void bitonic_rows(int32_t (&v)[E], int k)
{
#pragma unroll
    for (int r = 0; r < E; ++r) {
        const int rp = r ^ JR;
        if (rp > r) {
            const bool asc = ((r * 32) & k) == 0;
            const int32_t a = v[r], b = v[rp];
            const bool sw = asc ? (a > b) : (a < b);
            v[r] = sw ? b : a;
            v[rp] = sw ? a : b;
        }
    }
}
template <int E>
__device__ __forceinline__ void warp_bitonic_rolled(int32_t (&v)[E])
{
    static_assert(E == 16 || E == 32 || E == 64, "rolled network for 16, 32 or 64 rows");
    const int lane = threadIdx.x & 31;
    constexpr int P = 32 * E;
#pragma unroll 1
    for (int k = 2; k <= P; k <<= 1) {
#pragma unroll 1
        for (int j = k >> 1; j > 0; j >>= 1) {
            if (j >= 32) {
                switch (j >> 5) {
                case 1: bitonic_rows<1>(v, k); break;
                case 2: bitonic_rows<2>(v, k); break;
                case 4: bitonic_rows<4>(v, k); break;
                case 8: bitonic_rows<8>(v, k); break;
                default:
                    if constexpr (E >= 32) {
                        if (j >> 5 == 16) bitonic_rows<16>(v, k);
                        else if constexpr (E == 64) bitonic_rows<32>(v, k);
                    }
                    break;
                }
            } else {
                const bool lower = (lane & j) == 0;
#pragma unroll
                for (int r = 0; r < E; ++r) {
                    const int p = r * 32 + lane;
                    const int32_t o = __shfl_xor_sync(0xFFFFFFFFu, v[r], j);
                    const bool asc = (p & k) == 0;
                    v[r] = (lower == asc) ? min(v[r], o) : max(v[r], o);
                }
            }
        }
    }
}

// Batcher's odd-even merge sort of a[0, n) in global memory by one warp.
// Every comparator moves the smaller key to the lower index, so lengths that
// are not a power of two need no padding.
__device__ __forceinline__ void warp_oddeven_sort(int32_t* a, int n)
{
    const int lane = threadIdx.x & 31;
    for (int p = 1; p < n; p <<= 1) {
        for (int k = p; k >= 1; k >>= 1) {
            const int j0 = k % p;
            const int nblk = (n - j0 + 2 * k - 1) / (2 * k);
            for (int t = lane; t < nblk * k; t += 32) {
                const int b = t / k, i = t - b * k;
                const int lo = j0 + 2 * k * b + i, hi = lo + k;
                if (hi < n && (lo / (2 * p)) == (hi / (2 * p))) {
                    const int32_t x = a[lo], y = a[hi];
                    if (x > y) {
                        a[lo] = y;
                        a[hi] = x;
                    }
                }
            }
            __syncwarp();
        }
    }
}

__device__ __forceinline__ void copy_particle(const Cols& A, const Cols& B, int32_t src, int64_t dst)
{
    B.wv[dst] = ldg_pv(A.wv + src);
    B.pos[dst] = ldg_px(A.pos + src);
}

// B[start + q] = A[v[q]] (both records) for the warp's E register-major rows,
// in chunks of two rows whose loads are all issued before the chunk's
// stores: the gather is bound by the latency of these scattered reads, so
// they must be in flight together.  Plain loads keep each chunk's loads behind
// the previous chunk's stores, which bounds the registers in flight.
// Partial sums of the first props pass over one lane's particles
// (sum w, sum w v), accumulated in the order of props_cell's loop.
struct Sums4 {
    double n, sx, sy, sz;
};

template <int E>
__device__ __forceinline__ void gather_records(const Cols& A, const Cols& B, const int32_t (&v)[E], int32_t start,
                                               int32_t N, Sums4& acc)
{
    constexpr int CH = E < 2 ? E : 2;
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int r0 = 0; r0 < E; r0 += CH) {
        double2 t[CH][4];
#pragma unroll
        for (int r = 0; r < CH; ++r) {
            const bool in = ((r0 + r) * 32 + lane) < N;
            const double2* pv = reinterpret_cast<const double2*>(A.wv + (in ? v[r0 + r] : 0));
            const double2* px = reinterpret_cast<const double2*>(A.pos + (in ? v[r0 + r] : 0));
            t[r][0] = in ? pv[0] : make_double2(0.0, 0.0);
            t[r][1] = in ? pv[1] : make_double2(0.0, 0.0);
            t[r][2] = in ? px[0] : make_double2(0.0, 0.0);
            t[r][3] = in ? px[1] : make_double2(0.0, 0.0);
        }
#pragma unroll
        for (int r = 0; r < CH; ++r) {
            const int q = (r0 + r) * 32 + lane;
            if (q < N) {
                double2* ov = reinterpret_cast<double2*>(B.wv + start + q);
                double2* ox = reinterpret_cast<double2*>(B.pos + start + q);
                ov[0] = t[r][0];
                ov[1] = t[r][1];
                ox[0] = t[r][2];
                ox[1] = t[r][3];
                const double w = t[r][0].x;
                acc.n += w;
                acc.sx += t[r][0].y * w;
                acc.sy += t[r][1].x * w;
                acc.sz += t[r][1].y * w;
            }
        }
    }
}

template <int E, bool ROLLED = false>
__device__ __forceinline__ void sort_gather_regs(const SpeciesView& S, int32_t c, int32_t start, int32_t N, Sums4& acc)
{
    const int lane = threadIdx.x & 31;
    int32_t v[E];
#pragma unroll
    for (int r = 0; r < E; ++r) {
        const int q = r * 32 + lane;
        v[r] = q < N ? S.idx[start + q] : INT_MAX;
    }
    if constexpr (ROLLED && E >= 16) warp_bitonic_rolled<E>(v);
    else warp_bitonic<E>(v);
    gather_records<E>(S.A, S.B, v, start, N, acc);
#pragma unroll
    for (int r = 0; r < E; ++r) {
        const int q = r * 32 + lane;
        if (q < N) {
            S.cellB[start + q] = c;
            S.key[start + q] = c;
        }
    }
}

// 16-byte asynchronous copy global -> shared (cp.async, L2 only): the data in
// flight holds no registers, so one warp can have a whole cell's records in
// flight at once
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem)
{
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all()
{
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

// sort_gather_regs with the gather staged in shared memory: every lane issues
// the asynchronous copies of all its rows (64 bytes each) into `stage`
// (STAGE_ROWS records of 64 bytes), waits for them, then writes the rows to B
// with coalesced stores.  Each lane reads back only what it copied itself.
constexpr int STAGE_ROWS = 512;

template <int E>
__device__ __forceinline__ void sort_gather_staged(const SpeciesView& S, int32_t c, int32_t start, int32_t N,
                                                   Sums4& acc, double2* stage)
{
    const int lane = threadIdx.x & 31;
    int32_t v[E];
#pragma unroll
    for (int r = 0; r < E; ++r) {
        const int q = r * 32 + lane;
        v[r] = q < N ? S.idx[start + q] : INT_MAX;
    }
    warp_bitonic<E>(v);
#pragma unroll
    for (int r = 0; r < E; ++r) {
        const int q = r * 32 + lane;
        if (q < N) {
            const double2* pv = reinterpret_cast<const double2*>(S.A.wv + v[r]);
            const double2* px = reinterpret_cast<const double2*>(S.A.pos + v[r]);
            double2* o = stage + 4 * q;
            cp_async16(o, pv);
            cp_async16(o + 1, pv + 1);
            cp_async16(o + 2, px);
            cp_async16(o + 3, px + 1);
        }
    }
    cp_async_wait_all();
#pragma unroll
    for (int r = 0; r < E; ++r) {
        const int q = r * 32 + lane;
        if (q < N) {
            const double2* t = stage + 4 * q;
            const double2 a = t[0], b = t[1], x0 = t[2], x1 = t[3];
            double2* ov = reinterpret_cast<double2*>(S.B.wv + start + q);
            double2* ox = reinterpret_cast<double2*>(S.B.pos + start + q);
            ov[0] = a;
            ov[1] = b;
            ox[0] = x0;
            ox[1] = x1;
            const double w = a.x;
            acc.n += w;
            acc.sx += a.y * w;
            acc.sy += b.x * w;
            acc.sz += b.y * w;
            S.cellB[start + q] = c;
            S.key[start + q] = c;
        }
    }
}

// Segments above 512 particles take an out-of-line call, so the registers
// their 32-row sort needs do not raise the register count of every caller.
template <bool ROLLED>
static __device__ __noinline__ void sort_gather_regs_32(const SpeciesView& S, int32_t c, int32_t start, int32_t N,
                                                        Sums4& acc)
{
    sort_gather_regs<32, ROLLED>(S, c, start, N, acc);
}

// Segments of 1,025 .. 2,048 particles in kernels with registers to spare
// (BIG): 64 rows per lane, out of line like the 32-row form.
template <bool ROLLED>
static __device__ __noinline__ void sort_gather_regs_64(const SpeciesView& S, int32_t c, int32_t start, int32_t N,
                                                        Sums4& acc)
{
    sort_gather_regs<64, ROLLED>(S, c, start, N, acc);
}

// Other segments of more than 1,024 particles sort their source slots with
// Batcher's network: in a per-warp shared-memory buffer of SORT_SMEM_KEYS
// keys where the launch provides one, else in place in global memory.
constexpr int SORT_SMEM_KEYS = 2048;

// Sort the source slots of cell c's segment [start, start + N) and gather the
// particles from buffer A into the same positions of buffer B (one warp).
// Returns this lane's first-pass props sums of the gathered particles.
// ROLLED: the 32- and 64-row sorts with the rolled network (kernels that
// only gather; the fused step kernel keeps the unrolled one, whose call
// needs fewer registers saved around it).
template <bool BIG = false, bool ROLLED = false>
__device__ __forceinline__ Sums4 sort_gather_segment(const SpeciesView& S, int32_t c, int32_t start, int32_t N,
                                                     int32_t* sortbuf = nullptr)
{
    Sums4 acc{0.0, 0.0, 0.0, 0.0};
    if (N <= 0) return acc;
    if (N <= 32) sort_gather_regs<1>(S, c, start, N, acc);
    else if (N <= 64) sort_gather_regs<2>(S, c, start, N, acc);
    else if (N <= 128) sort_gather_regs<4>(S, c, start, N, acc);
    else if (N <= 256) sort_gather_regs<8>(S, c, start, N, acc);
    else if (N <= 512) sort_gather_regs<16, ROLLED>(S, c, start, N, acc);
    else if (N <= 1024) sort_gather_regs_32<ROLLED>(S, c, start, N, acc);
    else if (BIG && N <= 2048) sort_gather_regs_64<ROLLED>(S, c, start, N, acc);
    else {
        const bool shared = sortbuf && N <= SORT_SMEM_KEYS;
        int32_t* keys = shared ? sortbuf : S.idx + start;
        if (shared) {
            for (int q = (threadIdx.x & 31); q < N; q += 32) sortbuf[q] = S.idx[start + q];
            __syncwarp();
        }
        warp_oddeven_sort(keys, N);
        for (int q = (threadIdx.x & 31); q < N; q += 32) {
            const int64_t dst = (int64_t)start + q;
            copy_particle(S.A, S.B, keys[q], dst);
            S.cellB[dst] = c;
            S.key[dst] = c;
            const PV r = S.B.wv[dst];
            acc.n += r.w;
            acc.sx += r.vx * r.w;
            acc.sy += r.vy * r.w;
            acc.sz += r.vz * r.w;
        }
        __syncwarp();  // the buffer is reused by the warp's next segment
    }
    return acc;
}

// sort_gather_segment through a shared-memory stage of STAGE_ROWS records
// (segments above that size take the register path)
__device__ __forceinline__ Sums4 sort_gather_segment_staged(const SpeciesView& S, int32_t c, int32_t start, int32_t N,
                                                            double2* stage)
{
    Sums4 acc{0.0, 0.0, 0.0, 0.0};
    if (N <= 0) return acc;
    if (N <= 32) sort_gather_staged<1>(S, c, start, N, acc, stage);
    else if (N <= 64) sort_gather_staged<2>(S, c, start, N, acc, stage);
    else if (N <= 128) sort_gather_staged<4>(S, c, start, N, acc, stage);
    else if (N <= 256) sort_gather_staged<8>(S, c, start, N, acc, stage);
    else if (N <= STAGE_ROWS) sort_gather_staged<16>(S, c, start, N, acc, stage);
    else return sort_gather_segment(S, c, start, N);
    return acc;
}

}  // namespace mz
