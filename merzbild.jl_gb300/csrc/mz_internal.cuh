// Internal definitions shared by the merzgpu CUDA translation units.
//
// Device layout of one domain (n_cells cells x n_species species):
//   per species, two arrays of 32-byte records -- {w, vx, vy, vz} and
//   {x, y, z, unused}, one DRAM sector each -- in two buffers (A = live,
//   B = sort target), int32 `cell` (cell that owns the
//   slot in the current layout, -1 = dead slot), int32 `key` (cell the slot
//   moves to at the next sort), and a per-cell indexer {start1, n_group1,
//   start2, n_group2} that has the meaning of Merzbild's ParticleIndexer
//   (particles.jl:56-66) with 0-based slots.  A cell's logical particle list is
//   group1 followed by group2 (map_cont_index, particles.jl:364-366).
//
// Slots [0, high_water) are either live or dead.  The global order of live
// slots is: every cell's group1 in cell order, then every cell's group2 in cell
// order -- the order Merzbild's squash_pia! (particles.jl:622-682) produces --
// so a stable counting sort over slots reproduces sort_particles!
// (grid_sorting.jl:58-113) bit for bit.
#pragma once

#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>

#define MZ_MAX_SPECIES 4
#define MZ_WARP 32

namespace mz {

// ------------------------------------------------------------------ status
enum : int {
    ST_OK = 0,
    ST_CAPACITY = 1,      // append / reservation would exceed capacity
    ST_OUTSIDE_GRID = 2,  // particle position maps outside [0, n_cells)
    ST_MERGE_BINS = 4,    // octree bin scratch exhausted
    ST_SEGMENT = 8,       // sort segment too large for the sorting path
    ST_WALL_HITS = 16,    // wall-hit loop reached its iteration cap
    ST_TIMEOUT = 32,      // a bounded wait for another warp's data gave up
};

// ------------------------------------------------------------------ RNG
// Philox4x32-10 (Salmon et al., SC'11).  Stream layout (identical to the
// CPU restatement used by the tests): key = seed, counter = (block, a, b, tag<<28 | sub<<24 | step&0xFFFFFF).
enum : uint32_t { TAG_NCOLL = 0, TAG_CAND = 1, TAG_CONVECT = 2, TAG_MERGE = 3, TAG_SAMPLE = 4, TAG_SAMPLE_CELL = 5 };

__host__ __device__ inline void philox4x32_10(uint32_t& c0, uint32_t& c1, uint32_t& c2, uint32_t& c3, uint32_t k0,
                                              uint32_t k1)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
#ifdef __CUDA_ARCH__
        uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
#else
        uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0, hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
#endif
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
    }
}

struct Stream {
    uint32_t k0, k1, a, b, c3;
    uint32_t n;        // next draw number
    uint32_t blk;      // block held in buf (0xFFFFFFFF = none)
    uint32_t buf[4];

    __host__ __device__ inline void init(uint64_t seed, uint32_t tag, uint32_t sub, uint32_t step, uint32_t a_,
                                         uint32_t b_)
    {
        k0 = (uint32_t)seed;
        k1 = (uint32_t)(seed >> 32);
        a = a_;
        b = b_;
        c3 = ((tag & 0xFu) << 28) | ((sub & 0xFu) << 24) | (step & 0xFFFFFFu);
        n = 0;
        blk = 0xFFFFFFFFu;
    }
    __host__ __device__ inline uint64_t bits()
    {
        uint32_t bk = n >> 1, e = n & 1u;
        if (bk != blk) {
            uint32_t c0 = bk, c1 = a, c2 = b, cc3 = c3;
            philox4x32_10(c0, c1, c2, cc3, k0, k1);
            buf[0] = c0;
            buf[1] = c1;
            buf[2] = c2;
            buf[3] = cc3;
            blk = bk;
        }
        ++n;
        // constant indices keep buf in registers
        const uint32_t lo = e ? buf[2] : buf[0], hi = e ? buf[3] : buf[1];
        return (uint64_t)lo | ((uint64_t)hi << 32);
    }
    // draws 2 bk and 2 bk + 1 of the stream (bits() of those positions),
    // without touching the stream's position
    __host__ __device__ inline void block_bits(uint32_t bk, uint64_t& d0, uint64_t& d1) const
    {
        uint32_t c0 = bk, c1 = a, c2 = b, cc3 = c3;
        philox4x32_10(c0, c1, c2, cc3, k0, k1);
        d0 = (uint64_t)c0 | ((uint64_t)c1 << 32);
        d1 = (uint64_t)c2 | ((uint64_t)cc3 << 32);
    }
    // the 52-bit integer m of the next uniform U = m * 2^-52
    __host__ __device__ inline uint64_t u52() { return bits() >> 12; }
    // uniform in [0, 1), multiples of 2^-52: [1, 2) - 1 like Julia's rand(Float64)
    __host__ __device__ inline double uniform()
    {
        uint64_t m = 0x3FF0000000000000ull | (bits() >> 12);
#ifdef __CUDA_ARCH__
        return __longlong_as_double((long long)m) - 1.0;
#else
        double d;
        memcpy(&d, &m, sizeof d);
        return d - 1.0;
#endif
    }
};

// U = m * 2^-52 as a double (exact)
__device__ __forceinline__ double u52_to_double(uint64_t m)
{
    return __longlong_as_double((long long)(0x3FF0000000000000ull | m)) - 1.0;
}

// floor(U * n) for U = m * 2^-52 with the FP64 product's rounding, computed in
// integer arithmetic: the exact product m * n / 2^52 splits into an integer
// part and a 64-bit fraction.  The rounded FP64 product can only differ from
// the exact floor when the fraction lies within half an ulp of the next
// integer (for n < 2^31 half an ulp is at most 2^-23); only then is the FP64
// formula evaluated.
__device__ __forceinline__ int32_t floor_u52_times(uint64_t m, int32_t n)
{
    const uint64_t a = m << 12;  // U * 2^64
    const uint64_t hi = __umul64hi(a, (uint64_t)n);
    const uint64_t lo = a * (uint64_t)n;
    if (lo >= 0xFFFFFE0000000000ull) return (int32_t)floor(u52_to_double(m) * (double)n);
    return (int32_t)hi;
}

// approximate log2 of a positive normal double (FP32 accuracy, no FP64 pipe)
__device__ __forceinline__ float log2_pos(double x)
{
    const uint64_t b = (uint64_t)__double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7FF) - 1023;
    const float mf = __int_as_float(0x3F800000 | (int)((b >> 29) & 0x7FFFFF));
    return (float)e + __log2f(mf);
}

// approximate log2(m * 2^-52) for a 52-bit integer m (U == 0 -> -1e30)
__device__ __forceinline__ float log2_u52(uint64_t m)
{
    if (m == 0) return -1e30f;
    const int lz = __clzll((long long)m);
    const uint32_t top = lz == 63 ? 0u : (uint32_t)((m << (lz + 1)) >> 41);  // 23 bits after the leading one
    return (float)(63 - lz - 52) + __log2f(__int_as_float(0x3F800000 | (int)top));
}

// ------------------------------------------------------------------ data
struct Interaction {  // Interaction, collision_utils.jl:73-82
    double m_r, mu1, mu2, vhs_d, vhs_o, vhs_Tref, vhs_muref, vhs_factor;
};

struct __align__(32) PV {  // weight and velocity of one particle
    double w, vx, vy, vz;
};

struct __align__(32) PX {  // position of one particle (the fourth word is unused)
    double x, y, z, unused;
};

struct Cols {  // one buffer of a species: record arrays indexed by slot
    PV* wv;
    PX* pos;
};

// 32-byte record moves as two 16-byte accesses; ldg_* read through the
// read-only path (for buffers no thread writes during the kernel)
__device__ __forceinline__ PV ldg_pv(const PV* p)
{
    const double2* q = reinterpret_cast<const double2*>(p);
    const double2 a = __ldg(q), b = __ldg(q + 1);
    return PV{a.x, a.y, b.x, b.y};
}
__device__ __forceinline__ PX ldg_px(const PX* p)
{
    const double2* q = reinterpret_cast<const double2*>(p);
    const double2 a = __ldg(q), b = __ldg(q + 1);
    return PX{a.x, a.y, b.x, b.y};
}

struct Indexer {  // {start1, n_group1, start2, n_group2}, 0-based slots
    int32_t start1, n1, start2, n2;
};

struct SpeciesView {
    Cols A, B;
    int32_t* cell;      // owner cell of each slot in A, -1 = dead
    int32_t* key;       // destination cell for the next sort
    int32_t* cellB;     // scratch for the cell column during gathers
    int32_t* idx;       // sort: source slot of each destination slot
    int32_t* counts;    // per-cell counts (n_cells + 1)
    int32_t* fill;      // per-cell scatter cursors
    Indexer* ind;       // per cell
    int64_t capacity;
    double mass;
};

struct CollisionFactors {  // CollisionFactors, collision_ntc.jl:18-25 (device)
    double smax;
    int32_t n1, n2;
    int32_t n_coll, n_coll_performed, n_eq_w_coll_performed, n_split;
};

struct Counters {  // per launch, reduced on device
    unsigned long long candidates, accepted, splits, merges, wall_hits;
};

struct DomainView {
    int32_t n_cells, n_species;
    SpeciesView sp[MZ_MAX_SPECIES];
    Interaction inter[MZ_MAX_SPECIES * MZ_MAX_SPECIES];  // [s1 + ns * s2]
    const double* cell_V;      // cell volumes
    const uint64_t* cell_seed; // per-cell RNG key (serving), nullptr = domain seed
    const uint32_t* cell_rid;  // per-cell RNG id, nullptr = cell index
    const uint32_t* cell_step; // per-cell step offset, nullptr = 0
    CollisionFactors* cf;      // [(s1 + ns * s2) * n_cells + cell]
    const double2* trig;       // sector table of sincos_2pi_u52
    int* status;               // device status word (ST_* bits)
    Counters* counters;
    uint64_t seed;
};

__device__ inline uint64_t cell_seed(const DomainView& d, int c) { return d.cell_seed ? d.cell_seed[c] : d.seed; }
__device__ inline uint32_t cell_rid(const DomainView& d, int c) { return d.cell_rid ? d.cell_rid[c] : (uint32_t)c; }
__device__ inline uint32_t cell_step(const DomainView& d, int c, uint32_t step)
{
    return d.cell_step ? step - d.cell_step[c] : step;
}

// logical index j -> slot (map_cont_index, particles.jl:364-366)
__device__ inline int32_t map_slot(const Indexer& p, int32_t j) { return j < p.n1 ? p.start1 + j : p.start2 + (j - p.n1); }

__device__ inline unsigned lanemask_lt()
{
    unsigned m;
    asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// warp-aggregated atomicAdd of 1 to ctr[key]; returns this lane's ticket
__device__ inline int32_t warp_agg_ticket(int32_t* ctr, int32_t key, unsigned active)
{
    unsigned peers = __match_any_sync(active, key);
    int leader = __ffs(peers) - 1;
    int rank = __popc(peers & lanemask_lt());
    int32_t base = 0;
    if ((int)(threadIdx.x & 31) == leader) base = atomicAdd(&ctr[key], __popc(peers));
    base = __shfl_sync(peers, base, leader);
    return base + rank;
}

__device__ inline void warp_agg_add(int32_t* ctr, int32_t key, unsigned active)
{
    unsigned peers = __match_any_sync(active, key);
    int leader = __ffs(peers) - 1;
    if ((int)(threadIdx.x & 31) == leader) atomicAdd(&ctr[key], __popc(peers));
}

__device__ inline double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    return v;
}

// G consecutive lanes of a warp acting as one unit (G = 8, 16 or 32); the
// masks let groups of one warp run loops of different lengths.
template <int G>
struct WarpGroup {
    static_assert(G == 8 || G == 16 || G == 32, "group width");
    int rank;       // lane within the group
    int base;       // first lane of the group
    unsigned mask;  // lanes of the group
    __device__ __forceinline__ WarpGroup()
    {
        const int lane = threadIdx.x & 31;
        rank = lane & (G - 1);
        base = lane & ~(G - 1);
        mask = G == 32 ? 0xFFFFFFFFu : (((1u << G) - 1u) << base);
    }
    // bit r set when group rank r has p
    __device__ __forceinline__ unsigned ballot(bool p) const { return __ballot_sync(mask, p) >> base; }
    template <class T>
    __device__ __forceinline__ T shfl(T v, int src) const { return __shfl_sync(mask, v, src, G); }
    template <class T>
    __device__ __forceinline__ T up(T v, int o) const { return __shfl_up_sync(mask, v, o, G); }
    __device__ __forceinline__ void sync() const { __syncwarp(mask); }
};

__device__ inline void set_status(const DomainView& d, int bits)
{
    if (d.status) atomicOr(d.status, bits);
}

constexpr double K_B = 1.380649e-23;           // constants.jl:4
constexpr double TWOPI = 2.0 * 3.141592653589793;
constexpr double EPS = 2.220446049250313e-16;  // Julia eps()

// ------------------------------------------------------------------ trig
// sin and cos of 2 pi m 2^-52 for a 52-bit integer m (the angle 2 pi rand()
// of the scattering), table-driven (P. T. P. Tang, "Table-driven implementation
// of the sine and cosine functions", 1990, in its simplest form): the top 8
// bits of m pick a sector whose centre angle c_i has {sin, cos} tabulated as
// double-double; the offset d = 2 pi (m - centre) 2^-52, |d| <= pi / 256,
// enters through
//   sin d = d - d^3/6 + d^5/120 - d^7/5040      (next term < 2e-23)
//   cos d - 1 = -d^2/2 + d^4/24 - d^6/720        (next term < 5e-20)
// and the angle-addition formulas, with the small terms summed before the
// tabulated leading part so that one rounding of the result dominates.
// About 16 FP64 operations replace the range reduction and the two long
// polynomials of a general sincos; the error stays within 1.5 ulp of the exact
// sine and cosine of 2 pi m 2^-52 (a double-rounded 2 pi U fed to sin/cos
// already differs from it by up to 4 ulp).
constexpr int TRIG_SECTORS = 256;

// tab: 2 * TRIG_SECTORS entries, {sin, cos} leading parts at 2 i and
// trailing parts at 2 i + 1
__device__ __forceinline__ void sincos_2pi_u52(const double2* tab, uint64_t m, double& s, double& c)
{
    const int i = (int)(m >> 44);
    const long long t = (long long)(m & 0xFFFFFFFFFFFull) - (1ll << 43);
    const double dl = (double)t * (TWOPI * 0x1p-52);
    const double d2 = dl * dl;
    const double sd = fma(dl * d2, fma(d2, fma(d2, -1.0 / 5040.0, 1.0 / 120.0), -1.0 / 6.0), dl);
    const double cm1 = d2 * fma(d2, fma(d2, -1.0 / 720.0, 1.0 / 24.0), -0.5);
    const double2 hi = __ldg(tab + 2 * i);
    const double2 lo = __ldg(tab + 2 * i + 1);
    s = hi.x + fma(hi.y, sd, fma(hi.x, cm1, lo.x));
    c = hi.y + fma(-hi.x, sd, fma(hi.y, cm1, lo.y));
}

}  // namespace mz
