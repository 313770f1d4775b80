// Internal definitions shared by the merzgpu CUDA translation units.
//
// Device layout of one domain (n_cells cells x n_species species):
//   per species, structure-of-arrays FP64 columns w, vx, vy, vz, x, y, z in
//   two buffers (A = live, B = sort target), int32 `cell` (cell that owns the
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
        return (uint64_t)buf[2 * e] | ((uint64_t)buf[2 * e + 1] << 32);
    }
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

// ------------------------------------------------------------------ data
struct Interaction {  // Interaction, collision_utils.jl:73-82
    double m_r, mu1, mu2, vhs_d, vhs_o, vhs_Tref, vhs_muref, vhs_factor;
};

struct Cols {  // one SoA buffer of a species
    double *w, *vx, *vy, *vz, *x, *y, *z;
};

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

__device__ inline void set_status(const DomainView& d, int bits)
{
    if (d.status) atomicOr(d.status, bits);
}

constexpr double K_B = 1.380649e-23;           // constants.jl:4
constexpr double TWOPI = 2.0 * 3.141592653589793;
constexpr double EPS = 2.220446049250313e-16;  // Julia eps()

}  // namespace mz
