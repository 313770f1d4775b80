// N:2 octree merging -- merge_octree_N2_based! (merging_octree_N2.jl:1060-1094)
// with OctreeBinMidSplit, the three initial-bound rules and both bound rules,
// with or without the 1-D position clamp (compute_new_particles!, :736-933).
//
// One warp merges one cell; cells are independent, so a launch covers every
// selected cell.  The warp keeps the reference's octree exactly:
//   * the bin to split is the heaviest refinable one, first in bin order on
//     ties (compute_octree!, :998-1039), found by a warp arg-max;
//   * split_bin! (:503-633): octants and counts per particle in parallel; the
//     per-octant weight sums are accumulated sequentially in particle order
//     (one lane per octant, over the octant's range after the counting sort),
//     so bin weights -- which decide later splits -- carry the reference's
//     rounding; children are numbered as the reference
//     numbers them and the particle list is re-ordered with the reference's
//     counting sort (which reverses the order inside each octant);
//   * bin moments (compute_bin_props!, :646-700) are sequential sums, one
//     lane per bin; bins of more than WIDE_BIN particles are summed by the
//     whole warp (equal to the sequential sums to round-off);
//   * the k-th bin that holds more than two particles draws its six direction
//     signs from draws 6k .. 6k+5 of the cell's stream: the reference's
//     sequential draws in bin order.
// New particles overwrite the cell's first slots in logical order and the
// remaining ones are deleted from the end (delete_particle_end!,
// particles.jl:478-566): group 2 first, then group 1; deleted slots become dead.
//
// Each warp works in its own slice of a scratch buffer: the bins, the
// particle list, the octant of every particle, a copy of the particles in
// list order (bin moments read contiguous ranges) and the new particles.
#include "mz_host.h"

#include <algorithm>

using namespace mz;

namespace {

enum : int { INIT_MINMAX = 1, INIT_MINMAX_SYM = 2, INIT_C = 3 };
enum : int { BOUNDS_INHERIT = 1, BOUNDS_RECOMPUTE = 2 };

struct MergeBin {  // OctreeCell (merging_octree_N2.jl:49-59) + its range of the particle list
    double w;
    double vmin[3], vmax[3];
    int32_t np, start, end;  // [start, end] positions in the particle list
    int32_t depth;
    int32_t refinable;
    int32_t pad;
};

struct MergeArgs {
    int s;
    int cb, ce;
    int64_t threshold;
    int32_t target;
    mz_octree_params prm;
    int clamp;
    double min_x, max_x;
    uint32_t step;
    // per-warp scratch: stride in bytes and offsets of each array
    char* scratch;
    size_t stride, off_pis, off_tmp, off_w, off_tw, off_lv, off_lx, off_oct, off_ov, off_ox;
    int64_t* deleted;  // total particles deleted
    int64_t* merged;   // cells merged
    unsigned int* next;  // cell counter of the warps
    // fused step: the RNG step index in device memory (nullptr: `step`), an
    // abort word (nonzero: the step was abandoned before it changed any
    // particle, do nothing) and the particle count the scratch slices hold
    const uint32_t* step_ptr;
    const int* abort;
    int32_t nmax;
    int32_t min_n;  // warp kernel: cells of at most min_n particles are left to the block kernel
};

// Integer order keys of doubles: for doubles that are not NaN, x > m exactly
// when key(x) > key(m) as signed integers (-0.0 taken as +0.0).  Compares,
// minima and maxima on keys run on the integer pipe; the FP64 pipe retires
// one warp instruction per 64 cycles.
__device__ __forceinline__ long long order_key(double x)
{
    long long b = __double_as_longlong(x);
    if (b == (long long)0x8000000000000000ull) b = 0;
    return b ^ ((b >> 63) & 0x7FFFFFFFFFFFFFFFll);
}
__device__ __forceinline__ double of_order_key(long long k)
{
    return __longlong_as_double(k ^ ((k >> 63) & 0x7FFFFFFFFFFFFFFFll));
}
__device__ __forceinline__ long long warp_min_key(long long v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = min(v, (long long)__shfl_xor_sync(0xFFFFFFFFu, v, o));
    return v;
}
__device__ __forceinline__ long long warp_max_key(long long v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, (long long)__shfl_xor_sync(0xFFFFFFFFu, v, o));
    return v;
}
// the minimum / maximum velocity keys over lane-strided particles
struct KeyBounds {
    long long lo[3], hi[3];
    __device__ __forceinline__ KeyBounds()
    {
        for (int c = 0; c < 3; ++c) {
            lo[c] = order_key(9299792458.0);
            hi[c] = order_key(-9299792458.0);
        }
    }
    __device__ __forceinline__ void add(const PV& v)
    {
        const long long k[3] = {order_key(v.vx), order_key(v.vy), order_key(v.vz)};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            lo[c] = min(lo[c], k[c]);
            hi[c] = max(hi[c], k[c]);
        }
    }
    __device__ __forceinline__ void warp_reduce()
    {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            lo[c] = warp_min_key(lo[c]);
            hi[c] = warp_max_key(hi[c]);
        }
    }
};

// compute_octant (merging_octree_N2.jl:304-316), 0-based
__device__ __forceinline__ int octant_of(const PV& v, const double* mid)
{
    return (v.vx > mid[0] ? 1 : 0) + (v.vy > mid[1] ? 2 : 0) + (v.vz > mid[2] ? 4 : 0);
}

// bin_bounds_recompute! (:382-418): min / max of the velocities of list[bs, be]
// (a zero bound may come out as +0.0 where the reference keeps -0.0: no
// octant test or output depends on the sign of a zero bound)
__device__ __forceinline__ void bounds_of(const Cols& A, const int32_t* pis, int bs, int be, double* mn, double* mx)
{
    const int lane = threadIdx.x & 31;
    KeyBounds kb;
    for (int i = bs + lane; i <= be; i += 32) kb.add(A.wv[pis[i]]);
    kb.warp_reduce();
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        mn[c] = of_order_key(kb.lo[c]);
        mx[c] = of_order_key(kb.hi[c]);
    }
}

// compute_bin_props! (:646-700) of the bin list[bs, be]: mean velocity and
// position, and the standard deviations sqrt(sum w (v - vm)^2 / w) per
// component; sums in particle order by one lane
__device__ __forceinline__ void bin_moments_lane(const PV* lv, const PX* lx, int bs, int be, double inv_w, double* vm,
                                                 double* xm, double* sv, double* sx)
{
    double vs[3] = {0, 0, 0}, xs[3] = {0, 0, 0};
    for (int k = 0; k < 3; ++k) vm[k] = xm[k] = 0.0;
    for (int i = bs; i <= be; ++i) {
        const PV v = lv[i];
        const PX x = lx[i];
        vm[0] = vm[0] + v.w * v.vx;
        vm[1] = vm[1] + v.w * v.vy;
        vm[2] = vm[2] + v.w * v.vz;
        xm[0] = xm[0] + v.w * x.x;
        xm[1] = xm[1] + v.w * x.y;
        xm[2] = xm[2] + v.w * x.z;
    }
    for (int k = 0; k < 3; ++k) {
        vm[k] = vm[k] * inv_w;
        xm[k] = xm[k] * inv_w;
    }
    for (int i = bs; i <= be; ++i) {
        const PV v = lv[i];
        const PX x = lx[i];
        const double dv[3] = {v.vx - vm[0], v.vy - vm[1], v.vz - vm[2]};
        const double dx[3] = {x.x - xm[0], x.y - xm[1], x.z - xm[2]};
        for (int k = 0; k < 3; ++k) {
            vs[k] = vs[k] + v.w * (dv[k] * dv[k]);
            xs[k] = xs[k] + v.w * (dx[k] * dx[k]);
        }
    }
    for (int k = 0; k < 3; ++k) {
        sv[k] = sqrt(vs[k] * inv_w);
        sx[k] = sqrt(xs[k] * inv_w);
    }
}

__device__ __forceinline__ double warp_sum_d(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    return v;
}

// the same moments by the whole warp: lane-strided partial sums added in a
// tree (equal to the sequential sums to round-off; the bin weight inv_w and
// with it every split decision come from the sequential octant sums)
__device__ __forceinline__ void bin_moments_warp(const PV* lv, const PX* lx, int bs, int be, double inv_w, double* vm,
                                                 double* xm, double* sv, double* sx)
{
    const int lane = threadIdx.x & 31;
    double m[6] = {0, 0, 0, 0, 0, 0};
    for (int i = bs + lane; i <= be; i += 32) {
        const PV v = lv[i];
        const PX x = lx[i];
        m[0] += v.w * v.vx;
        m[1] += v.w * v.vy;
        m[2] += v.w * v.vz;
        m[3] += v.w * x.x;
        m[4] += v.w * x.y;
        m[5] += v.w * x.z;
    }
    for (int k = 0; k < 3; ++k) {
        vm[k] = warp_sum_d(m[k]) * inv_w;
        xm[k] = warp_sum_d(m[3 + k]) * inv_w;
    }
    double q[6] = {0, 0, 0, 0, 0, 0};
    for (int i = bs + lane; i <= be; i += 32) {
        const PV v = lv[i];
        const PX x = lx[i];
        const double dv[3] = {v.vx - vm[0], v.vy - vm[1], v.vz - vm[2]};
        const double dx[3] = {x.x - xm[0], x.y - xm[1], x.z - xm[2]};
        for (int k = 0; k < 3; ++k) {
            q[k] += v.w * (dv[k] * dv[k]);
            q[3 + k] += v.w * (dx[k] * dx[k]);
        }
    }
    for (int k = 0; k < 3; ++k) {
        sv[k] = sqrt(warp_sum_d(q[k]) * inv_w);
        sx[k] = sqrt(warp_sum_d(q[3 + k]) * inv_w);
    }
}

// compute_new_particles! (:736-933) for one bin of more than two particles:
// two particles of half its weight at vm -/+ sv and xm -/+ sx, the six signs
// from draws 6k .. 6k+5 of the cell's stream (k-th such bin), positions
// clamped to the grid in 1-D
__device__ __forceinline__ void emit_pair(const MergeArgs& a, const Stream& st, int kbig, double w,
                                          const double* vm, const double* xm, const double* sv, const double* sx,
                                          PV* ov, PX* ox)
{
    Stream r = st;
    r.n = 6u * (uint32_t)kbig;
    double dvs[3], dxs[3];
    for (int k = 0; k < 3; ++k) dvs[k] = r.u52() < (1ull << 51) ? -1.0 : 1.0;
    for (int k = 0; k < 3; ++k) dxs[k] = r.u52() < (1ull << 51) ? -1.0 : 1.0;
    const double w1 = 0.5 * w;
    double x1[3], x2[3];
    for (int k = 0; k < 3; ++k) {
        x1[k] = xm[k] + dxs[k] * sx[k];
        x2[k] = xm[k] - dxs[k] * sx[k];
    }
    if (a.clamp) {
        x1[0] = x1[0] < a.min_x ? a.min_x : (x1[0] > a.max_x ? a.max_x : x1[0]);
        x2[0] = x2[0] < a.min_x ? a.min_x : (x2[0] > a.max_x ? a.max_x : x2[0]);
    }
    ov[0] = PV{w1, vm[0] + dvs[0] * sv[0], vm[1] + dvs[1] * sv[1], vm[2] + dvs[2] * sv[2]};
    ov[1] = PV{w1, vm[0] - dvs[0] * sv[0], vm[1] - dvs[1] * sv[1], vm[2] - dvs[2] * sv[2]};
    ox[0] = PX{x1[0], x1[1], x1[2], 0.0};
    ox[1] = PX{x2[0], x2[1], x2[2], 0.0};
}

constexpr int WIDE_BIN = 48;  // bins of more particles get their moments from the whole warp

__device__ void merge_cell(const DomainView& d, const MergeArgs& a, int c, char* base)
{
    const int lane = threadIdx.x & 31;
    const SpeciesView& S = d.sp[a.s];
    const Cols& A = S.A;
    MergeBin* bins = reinterpret_cast<MergeBin*>(base);
    int32_t* pis = reinterpret_cast<int32_t*>(base + a.off_pis);
    int32_t* tmp = reinterpret_cast<int32_t*>(base + a.off_tmp);
    double* wl = reinterpret_cast<double*>(base + a.off_w);
    double* tw = reinterpret_cast<double*>(base + a.off_tw);
    PV* lv = reinterpret_cast<PV*>(base + a.off_lv);
    PX* lx = reinterpret_cast<PX*>(base + a.off_lx);
    uint8_t* oct = reinterpret_cast<uint8_t*>(base + a.off_oct);
    PV* ov = reinterpret_cast<PV*>(base + a.off_ov);
    PX* ox = reinterpret_cast<PX*>(base + a.off_ox);
    const Indexer p = S.ind[c];
    const int n = p.n1 + p.n2;

    // init_octree! (:947-984)
    for (int i = lane; i < n; i += 32) pis[i] = map_slot(p, i);
    __syncwarp();
    double mn[3], mx[3];
    if (a.prm.init_bin_bounds == INIT_C) {
        for (int k = 0; k < 3; ++k) {
            mn[k] = -299792458.0;
            mx[k] = 299792458.0;
        }
    } else {
        bounds_of(A, pis, 0, n - 1, mn, mx);
        if (a.prm.init_bin_bounds == INIT_MINMAX_SYM)
            for (int k = 0; k < 3; ++k) {
                const double m = fmax(fabs(mn[k]), fabs(mx[k]));
                mn[k] = -m;
                mx[k] = m;
            }
    }
    if (lane == 0) {
        MergeBin b;
        b.w = 1e50;
        for (int k = 0; k < 3; ++k) {
            b.vmin[k] = mn[k];
            b.vmax[k] = mx[k];
        }
        b.np = n;
        b.start = 0;
        b.end = n - 1;
        b.depth = 0;
        b.refinable = (n > 2) && (a.prm.max_depth > 0);
        b.pad = 0;
        bins[0] = b;
    }
    int nbins = 1;
    int total = n >= 2 ? 2 : n;  // total_post_merge_np
    __syncwarp();

    // compute_octree! (:998-1039)
    for (;;) {
        double bw = -1.0;
        int bid = -1;
        for (int b = lane; b < nbins; b += 32) {
            const MergeBin& B = bins[b];
            if (B.refinable && B.w > bw) {
                bw = B.w;
                bid = b;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double w2 = __shfl_xor_sync(0xFFFFFFFFu, bw, o);
            const int id2 = __shfl_xor_sync(0xFFFFFFFFu, bid, o);
            if (id2 >= 0 && (bid < 0 || w2 > bw || (w2 == bw && id2 < bid))) {
                bw = w2;
                bid = id2;
            }
        }
        if (bid < 0) break;
        if (total + 14 > a.target) break;

        // split_bin! (:503-633)
        const MergeBin P = bins[bid];
        const int bs = P.start, be = P.end, nb = be - bs + 1;
        double vmin[3], vmax[3];
        for (int k = 0; k < 3; ++k) {
            vmin[k] = P.vmin[k];
            vmax[k] = P.vmax[k];
        }
        if (a.prm.bin_bounds_compute == BOUNDS_RECOMPUTE) bounds_of(A, pis, bs, be, vmin, vmax);
        double mid[3];
        for (int k = 0; k < 3; ++k) mid[k] = 0.5 * (vmin[k] + vmax[k]);
        // octant and weight of every particle, in parallel
        int cnt[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int i = lane; i < nb; i += 32) {
            const PV v = A.wv[pis[bs + i]];
            const int o = octant_of(v, mid);
            oct[i] = (uint8_t)o;
            wl[i] = v.w;
#pragma unroll
            for (int k = 0; k < 8; ++k) cnt[k] += (o == k);
        }
#pragma unroll
        for (int k = 0; k < 8; ++k) cnt[k] = __reduce_add_sync(0xFFFFFFFFu, cnt[k]);
        __syncwarp();
        int incl[8], run = 0;
        int nne = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            run += cnt[k];
            incl[k] = run;
            nne += cnt[k] > 0;
        }
        // the reference's counting sort: octant k fills [incl[k-1], incl[k])
        // from its end, in particle order
        int seen[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int i0 = 0; i0 < nb; i0 += 32) {
            const int i = i0 + lane;
            const bool in = i < nb;
            const int o = in ? oct[i] : 8;
            const unsigned peers = __match_any_sync(0xFFFFFFFFu, o);
            int r = __popc(peers & lanemask_lt()), end_o = 0;
#pragma unroll
            for (int k = 0; k < 8; ++k)
                if (o == k) {
                    r += seen[k];
                    end_o = incl[k];
                }
            if (in) {
                tmp[end_o - 1 - r] = pis[bs + i];
                tw[end_o - 1 - r] = wl[i];
            }
#pragma unroll
            for (int k = 0; k < 8; ++k) seen[k] += __popc(__ballot_sync(0xFFFFFFFFu, in && o == k));
        }
        // weight per octant, summed in particle order as the reference sums
        // it: octant k's particles now sit in [incl[k-1], incl[k]) in reversed
        // particle order, so lane k walks that range backwards
        __syncwarp();
        double wo = 0.0;
        {
            int lo = 0, hi = 0;
#pragma unroll
            for (int k = 0; k < 8; ++k)
                if (lane == k) {
                    lo = incl[k] - cnt[k];
                    hi = incl[k];
                }
            for (int j = hi - 1; j >= lo; --j) wo += tw[j];
        }
        // children: non-empty octants in order; the first keeps the bin id
        {
            int kch = 0, startk = bs;
            for (int k = 0; k < 8; ++k) {
                if (cnt[k] == 0) continue;
                const int id = kch == 0 ? bid : nbins + kch - 1;
                const double wk = __shfl_sync(0xFFFFFFFFu, wo, k);
                if (lane == 0) {
                    MergeBin b;
                    for (int q = 0; q < 3; ++q) {
                        const bool upper = (k >> q) & 1;
                        if (a.prm.bin_bounds_compute == BOUNDS_INHERIT) {
                            // bin_bounds_inherit! (:341-367)
                            b.vmin[q] = upper ? mid[q] : P.vmin[q];
                            b.vmax[q] = upper ? P.vmax[q] : mid[q];
                        } else {
                            b.vmin[q] = P.vmin[q];
                            b.vmax[q] = P.vmax[q];
                        }
                    }
                    b.np = cnt[k];
                    b.w = wk;
                    b.depth = P.depth + 1;
                    b.start = startk;
                    b.end = startk + cnt[k] - 1;
                    b.refinable = (cnt[k] > 2) && (b.depth < a.prm.max_depth);
                    b.pad = 0;
                    bins[id] = b;
                }
                total += cnt[k] >= 2 ? 2 : cnt[k];
                startk += cnt[k];
                ++kch;
            }
            total -= 2;
        }
        __syncwarp();
        for (int i = lane; i < nb; i += 32) pis[bs + i] = tmp[i];
        nbins += nne - 1;
        __syncwarp();
        if (nbins + 7 > a.prm.max_Nbins) break;
    }
    // the particles in list order, so that every bin reads a contiguous range
    for (int i = lane; i < n; i += 32) {
        lv[i] = A.wv[pis[i]];
        lx[i] = A.pos[pis[i]];
    }
    __syncwarp();
    if (nbins == 1 && lane == 0) {
        double w = 0.0;
        for (int i = 0; i < n; ++i) w += lv[i].w;
        bins[0].w = w;
    }
    __syncwarp();

    // compute_bin_props! (:646-700) and compute_new_particles! (:736-933),
    // one lane per bin (the whole warp for bins of many particles); outputs
    // in bin order
    int out_base = 0, big_base = 0;
    Stream st;
    st.init(cell_seed(d, c), TAG_MERGE, (uint32_t)a.s, cell_step(d, c, a.step), cell_rid(d, c), 0);
    for (int b0 = 0; b0 < nbins; b0 += 32) {
        const int b = b0 + lane;
        MergeBin B;
        int npe = 0;
        if (b < nbins) {
            B = bins[b];
            npe = B.w == 0.0 ? 0 : B.np;
        }
        const int cnt_out = npe >= 2 ? 2 : npe;
        const int big = npe > 2 ? 1 : 0;
        int io = cnt_out, ib = big;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t1 = __shfl_up_sync(0xFFFFFFFFu, io, o);
            const int t2 = __shfl_up_sync(0xFFFFFFFFu, ib, o);
            if (lane >= o) {
                io += t1;
                ib += t2;
            }
        }
        const int pos = out_base + io - cnt_out, kbig = big_base + ib - big;
        const bool wide = npe > WIDE_BIN;
        if (npe > 2 && !wide) {
            double vm[3], xm[3], sv[3], sx[3];
            bin_moments_lane(lv, lx, B.start, B.end, 1.0 / B.w, vm, xm, sv, sx);
            emit_pair(a, st, kbig, B.w, vm, xm, sv, sx, ov + pos, ox + pos);
        } else if (npe >= 1 && npe <= 2) {
            // np == 1 or 2: the bin's particles are kept as they are
            for (int q = 0; q < npe; ++q) {
                ov[pos + q] = lv[B.start + q];
                ox[pos + q] = lx[B.start + q];
            }
        }
        // bins of many particles: the whole warp sums their moments, one bin
        // at a time (a lane alone would walk hundreds of particles)
        unsigned wmask = __ballot_sync(0xFFFFFFFFu, wide);
        while (wmask) {
            const int q = __ffs(wmask) - 1;
            wmask &= wmask - 1;
            const int qs = __shfl_sync(0xFFFFFFFFu, B.start, q), qe = __shfl_sync(0xFFFFFFFFu, B.end, q);
            const double qw = __shfl_sync(0xFFFFFFFFu, B.w, q);
            const int qpos = __shfl_sync(0xFFFFFFFFu, pos, q), qk = __shfl_sync(0xFFFFFFFFu, kbig, q);
            double vm[3], xm[3], sv[3], sx[3];
            bin_moments_warp(lv, lx, qs, qe, 1.0 / qw, vm, xm, sv, sx);
            if (lane == 0) emit_pair(a, st, qk, qw, vm, xm, sv, sx, ov + qpos, ox + qpos);
        }
        out_base += __shfl_sync(0xFFFFFFFFu, io, 31);
        big_base += __shfl_sync(0xFFFFFFFFu, ib, 31);
    }
    __syncwarp();
    const int cur = out_base;
    for (int j = lane; j < cur; j += 32) {
        const int32_t slot = map_slot(p, j);
        A.wv[slot] = ov[j];
        A.pos[slot] = ox[j];
    }
    for (int j = cur + lane; j < n; j += 32) {
        const int32_t slot = map_slot(p, j);
        A.wv[slot].w = 0.0;
        S.cell[slot] = -1;
    }
    if (lane == 0) {
        Indexer q = p;
        if (cur <= p.n1) {
            q.n1 = cur;
            q.n2 = 0;
            q.start2 = 0;
            if (cur == 0) q.start1 = 0;
        } else {
            q.n2 = cur - p.n1;
        }
        S.ind[c] = q;
        if (n > cur) atomicAdd((unsigned long long*)a.deleted, (unsigned long long)(n - cur));
        atomicAdd((unsigned long long*)a.merged, 1ull);
        atomicAdd(&d.counters->merges, 1ull);
    }
}

// Warps take the next cell from a counter, so the merged cells (a minority of
// the range, and each merge a long chain) spread evenly over the warps.
__global__ void __launch_bounds__(256) k_merge(DomainView d, MergeArgs a)
{
    if (a.abort && *a.abort) return;
    if (a.step_ptr) a.step = *a.step_ptr;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    char* base = a.scratch + (size_t)warp * a.stride;
    for (;;) {
        // lane 0 claims cells until it finds one to merge
        int c = a.ce;
        if (lane == 0)
            for (;;) {
                const int q = a.cb + (int)atomicAdd(a.next, 1u);
                if (q >= a.ce) break;
                const Indexer p = d.sp[a.s].ind[q];
                const int n = p.n1 + p.n2;
                if (n > a.min_n && (a.threshold < 0 || n > a.threshold)) {
                    if (n > a.nmax) {  // larger than the scratch slices: leave the cell
                        set_status(d, ST_CAPACITY);
                        continue;
                    }
                    c = q;
                    break;
                }
            }
        c = __shfl_sync(0xFFFFFFFFu, c, 0);
        if (c >= a.ce) break;
        merge_cell(d, a, c, base);
        __syncwarp();
    }
}

// ---------------------------------------------------------------- block form
// A cell of up to MB_N particles (target at most MB_BINS) merges in one block
// of MB_THREADS threads with its particles, lists and bins in shared memory:
// the particles are staged once in logical order (cv), the octree is built by
// the first warp exactly as merge_cell builds it (indices into cv instead of
// slots), and the parallel parts -- staging, bounds, the list-order copy, the
// bin moments (one thread per bin, the wide bins one warp each) and the write-
// back -- use every warp.  Same arithmetic in the same order as merge_cell.
constexpr int MB_THREADS = 256, MB_N = 1536, MB_BINS = 384;
constexpr int MB_SPLIT_BLOCK = 128;  // splits of at least this many particles run on every warp of the block
constexpr size_t MB_OFF_PIS = (size_t)MB_BINS * sizeof(MergeBin);
constexpr size_t MB_OFF_CV = MB_OFF_PIS + (size_t)MB_N * sizeof(int32_t);
constexpr size_t MB_OFF_LV = MB_OFF_CV + (size_t)MB_N * sizeof(PV);
constexpr size_t MB_OFF_R = MB_OFF_LV + (size_t)MB_N * sizeof(PV);  // lx; during the octree tmp, wl, tw, oct
constexpr size_t MB_OFF_OV = MB_OFF_R + (size_t)MB_N * sizeof(PX);
constexpr size_t MB_OFF_OX = MB_OFF_OV + (size_t)MB_BINS * sizeof(PV);
constexpr size_t MB_SMEM = MB_OFF_OX + (size_t)MB_BINS * sizeof(PX);
static_assert((size_t)MB_N * (sizeof(int32_t) + 2 * sizeof(double) + 1) <= (size_t)MB_N * sizeof(PX),
              "octree scratch must fit the position region");

// FP32 value of a positive double by truncation of its mantissa (relative
// error below 2^-23, never upward); ok = false outside the FP32 normal range
__device__ __forceinline__ float f32_of_positive(double x, bool& ok)
{
    const long long bits = __double_as_longlong(x);
    if (bits == 0) {
        ok = true;
        return 0.0f;
    }
    const int e = (int)((bits >> 52) & 0x7FF) - 1023;
    ok = bits > 0 && e >= -126 && e <= 127;
    return __int_as_float(((e + 127) << 23) | (int)((bits >> 29) & 0x7FFFFF));
}

// compute_octant through integer keys
__device__ __forceinline__ int octant_of_keys(const PV& v, const long long* km)
{
    return (order_key(v.vx) > km[0] ? 1 : 0) + (order_key(v.vy) > km[1] ? 2 : 0) + (order_key(v.vz) > km[2] ? 4 : 0);
}

__device__ __forceinline__ void bounds_of_list(const PV* cv, const int32_t* pis, int bs, int be, double* mn,
                                               double* mx)
{
    const int lane = threadIdx.x & 31;
    KeyBounds kb;
    for (int i = bs + lane; i <= be; i += 32) kb.add(cv[pis[i]]);
    kb.warp_reduce();
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        mn[c] = of_order_key(kb.lo[c]);
        mx[c] = of_order_key(kb.hi[c]);
    }
}

__device__ void merge_cell_block(const DomainView& d, const MergeArgs& a, int c, char* smem)
{
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int NW = MB_THREADS / 32;
    const SpeciesView& S = d.sp[a.s];
    const Cols& A = S.A;
    MergeBin* bins = reinterpret_cast<MergeBin*>(smem);
    int32_t* pis = reinterpret_cast<int32_t*>(smem + MB_OFF_PIS);
    PV* cv = reinterpret_cast<PV*>(smem + MB_OFF_CV);
    PV* lv = reinterpret_cast<PV*>(smem + MB_OFF_LV);
    PX* lx = reinterpret_cast<PX*>(smem + MB_OFF_R);
    int32_t* tmp = reinterpret_cast<int32_t*>(smem + MB_OFF_R);
    double* wl = reinterpret_cast<double*>(smem + MB_OFF_R + (size_t)MB_N * sizeof(int32_t));
    double* tw = wl + MB_N;
    uint8_t* oct = reinterpret_cast<uint8_t*>(tw + MB_N);
    PV* ov = reinterpret_cast<PV*>(smem + MB_OFF_OV);
    PX* ox = reinterpret_cast<PX*>(smem + MB_OFF_OX);
    __shared__ long long s_wk[MB_BINS];  // bin weights for the choice of the bin to split (see below)
    __shared__ int s_nbins;
    __shared__ int s_pos[MB_BINS], s_kbig[MB_BINS];
    __shared__ int s_scan[NW][2];
    const Indexer p = S.ind[c];
    const int n = p.n1 + p.n2;

    // init_octree! (:947-984): the cell's particles in logical order
    for (int i = tid; i < n; i += MB_THREADS) {
        cv[i] = A.wv[map_slot(p, i)];
        pis[i] = i;
    }
    __syncthreads();
    double mn[3], mx[3];
    if (a.prm.init_bin_bounds == INIT_C) {
        for (int k = 0; k < 3; ++k) {
            mn[k] = -299792458.0;
            mx[k] = 299792458.0;
        }
    } else {
        KeyBounds kb;
        for (int i = tid; i < n; i += MB_THREADS) kb.add(cv[i]);
        kb.warp_reduce();
        __shared__ long long s_kb[NW][6];
        if (lane == 0)
            for (int k = 0; k < 3; ++k) {
                s_kb[warp][k] = kb.lo[k];
                s_kb[warp][3 + k] = kb.hi[k];
            }
        __syncthreads();
        for (int k = 0; k < 3; ++k) {
            long long l = s_kb[0][k], h = s_kb[0][3 + k];
            for (int w = 1; w < NW; ++w) {
                l = min(l, s_kb[w][k]);
                h = max(h, s_kb[w][3 + k]);
            }
            mn[k] = of_order_key(l);
            mx[k] = of_order_key(h);
        }
        if (a.prm.init_bin_bounds == INIT_MINMAX_SYM)
            for (int k = 0; k < 3; ++k) {
                const double m = fmax(fabs(mn[k]), fabs(mx[k]));
                mn[k] = -m;
                mx[k] = m;
            }
    }

    {
        // compute_octree! (:998-1039).  The first warp chooses the bins to split
        // and writes the children.  A split of MB_SPLIT_BLOCK or more particles
        // runs its octant and counting-sort passes on every warp of the block,
        // each on a contiguous chunk of the bin's list (the counting sort's order
        // is the one-warp order: a warp's ranks start after the earlier chunks'),
        // smaller splits on the first warp alone.  The chosen bin and its
        // particle count pass through s_bid / s_nb by iteration parity: the
        // first warp writes a slot again only after every warp has passed the
        // next barrier, that is after each warp has read it.
        __shared__ int s_bid[2], s_nb[2];
        int it = 0;
        __shared__ int s_wc[NW][8];
        __shared__ float s_wf[NW][8];
        __shared__ int s_fok[NW];
        int nbins = 1;               // first warp
        int total = n >= 2 ? 2 : n;  // total_post_merge_np, first warp
        bool more = true;            // first warp: max_Nbins leaves room for a split
        if (warp == 0) {
            if (lane == 0) {
                MergeBin b;
                b.w = 1e50;
                for (int k = 0; k < 3; ++k) {
                    b.vmin[k] = mn[k];
                    b.vmax[k] = mx[k];
                }
                b.np = n;
                b.start = 0;
                b.end = n - 1;
                b.depth = 0;
                b.refinable = (n > 2) && (a.prm.max_depth > 0);
                b.pad = 0;
                bins[0] = b;
                s_wk[0] = b.refinable ? __double_as_longlong(1e50) : -1ll;
            }
            __syncwarp();
        }
        for (;;) {
            if (warp == 0) {
                // The heaviest refinable bin, first in bin order on ties.  A
                // child's weight -- the sum of its particles' weights in particle
                // order, the reference's rounding -- is a sequential FP64 chain;
                // here a child first gets an FP32 sum (within 4e-6 relative of the
                // exact one) and the choice is made on those when no other
                // refinable bin comes within 1e-5 of the largest; otherwise the
                // exact weights of the contenders decide.  Exact weights of the
                // remaining bins follow the octree, in parallel.  s_wk holds the
                // approximate weight of a refinable bin as the bits of the double
                // and -1 for the others: weights are not negative, and the bits of
                // non-negative doubles order as their values, so the choice runs
                // on integer compares (the FP64 pipe retires one warp instruction
                // per 64 cycles).  One pass yields the largest weight, its bin and
                // the runner-up weight.
                int bid = -1;
                if (more) {
                    long long k1 = -1, k2 = -1;
                    for (int b = lane; b < nbins; b += 32) {
                        const long long k = s_wk[b];
                        if (k > k1) {
                            k2 = k1;
                            k1 = k;
                            bid = b;
                        } else if (k > k2) {
                            k2 = k;
                        }
                    }
    #pragma unroll
                    for (int o = 16; o > 0; o >>= 1) {
                        const long long o1 = __shfl_xor_sync(0xFFFFFFFFu, k1, o);
                        const long long o2 = __shfl_xor_sync(0xFFFFFFFFu, k2, o);
                        const int oid = __shfl_xor_sync(0xFFFFFFFFu, bid, o);
                        const bool take = oid >= 0 && (bid < 0 || o1 > k1 || (o1 == k1 && oid < bid));
                        const long long lose = take ? k1 : o1;
                        k2 = max(max(k2, o2), lose);
                        if (take) {
                            k1 = o1;
                            bid = oid;
                        }
                    }
                    if (bid >= 0) {
                        const double b1 = __longlong_as_double(k1);
                        const long long kthr = __double_as_longlong(b1 - 1e-5 * b1);
                        if (k2 >= kthr) {
                            // the contenders' exact weights, then the heaviest of them
                            for (int b = lane; b < nbins; b += 32) {
                                MergeBin& B = bins[b];
                                if (s_wk[b] >= kthr && B.w < 0.0) {
                                    double w = 0.0;
                                    for (int j = B.end; j >= B.start; --j) w += cv[pis[j]].w;
                                    B.w = w;
                                }
                            }
                            __syncwarp();
                            long long bw = -1;
                            bid = -1;
                            for (int b = lane; b < nbins; b += 32) {
                                if (s_wk[b] < kthr) continue;
                                const long long w = __double_as_longlong(bins[b].w);
                                if (w > bw) {
                                    bw = w;
                                    bid = b;
                                }
                            }
    #pragma unroll
                            for (int o = 16; o > 0; o >>= 1) {
                                const long long w2 = __shfl_xor_sync(0xFFFFFFFFu, bw, o);
                                const int id2 = __shfl_xor_sync(0xFFFFFFFFu, bid, o);
                                if (id2 >= 0 && (bid < 0 || w2 > bw || (w2 == bw && id2 < bid))) {
                                    bw = w2;
                                    bid = id2;
                                }
                            }
                        }
                        if (total + 14 > a.target) bid = -1;
                    }
                }
                if (lane == 0) {
                    s_bid[it & 1] = bid;
                    s_nb[it & 1] = bid >= 0 ? bins[bid].end - bins[bid].start + 1 : 0;
                }
            }
            __syncthreads();
            const int bid = s_bid[it & 1], nb = s_nb[it & 1];
            ++it;
            if (bid < 0) break;
            const bool wide = nb >= MB_SPLIT_BLOCK;
            if (!wide && warp != 0) continue;  // the first warp splits alone

            // split_bin! (:503-633)
            const MergeBin P = bins[bid];
            const int bs = P.start, be = P.end;
            double vmin[3], vmax[3];
            for (int k = 0; k < 3; ++k) {
                vmin[k] = P.vmin[k];
                vmax[k] = P.vmax[k];
            }
            if (a.prm.bin_bounds_compute == BOUNDS_RECOMPUTE) bounds_of_list(cv, pis, bs, be, vmin, vmax);
            double mid[3];
            long long kmid[3];
            for (int k = 0; k < 3; ++k) {
                mid[k] = 0.5 * (vmin[k] + vmax[k]);
                kmid[k] = order_key(mid[k]);
            }
            // this warp's chunk of the list: all of it on the first warp alone
            const int chunk = wide ? ((nb + MB_THREADS - 1) / MB_THREADS) * 32 : nb;
            const int i0w = wide ? min(nb, warp * chunk) : 0;
            const int i1w = min(nb, i0w + chunk);
            // octants and counts; the octants' weights in FP32 on the way
            // (lane-strided partial sums of at most MB_N / 32 = 48 terms, a warp
            // tree, and the warps' sums added in warp order)
            int cnt[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            float wf[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            bool fok = true;
            for (int i = i0w + lane; i < i1w; i += 32) {
                const PV v = cv[pis[bs + i]];
                const int o = octant_of_keys(v, kmid);
                oct[i] = (uint8_t)o;
                wl[i] = v.w;
                bool ok;
                const float f = f32_of_positive(v.w, ok);
                fok &= ok;
    #pragma unroll
                for (int k = 0; k < 8; ++k) {
                    cnt[k] += (o == k);
                    if (o == k) wf[k] += f;
                }
            }
    #pragma unroll
            for (int k = 0; k < 8; ++k) {
                cnt[k] = __reduce_add_sync(0xFFFFFFFFu, cnt[k]);
    #pragma unroll
                for (int o = 16; o > 0; o >>= 1) wf[k] += __shfl_xor_sync(0xFFFFFFFFu, wf[k], o);
            }
            bool approx = __all_sync(0xFFFFFFFFu, fok);
            int seen[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            if (wide) {
                if (lane == 0) {
    #pragma unroll
                    for (int k = 0; k < 8; ++k) {
                        s_wc[warp][k] = cnt[k];
                        s_wf[warp][k] = wf[k];
                    }
                    s_fok[warp] = approx ? 1 : 0;
                }
                __syncthreads();
                // the bin's counts, and this warp's ranks start after the earlier chunks'
    #pragma unroll
                for (int k = 0; k < 8; ++k) {
                    int t = 0, before = 0;
                    float f = 0.f;
                    for (int w = 0; w < NW; ++w) {
                        const int x = s_wc[w][k];
                        t += x;
                        before += w < warp ? x : 0;
                        f += s_wf[w][k];
                    }
                    cnt[k] = t;
                    seen[k] = before;
                    wf[k] = f;
                }
                for (int w = 0; w < NW; ++w) approx &= s_fok[w] != 0;
            }
            __syncwarp();
            int incl[8], run = 0;
            int nne = 0;
    #pragma unroll
            for (int k = 0; k < 8; ++k) {
                run += cnt[k];
                incl[k] = run;
                nne += cnt[k] > 0;
            }
            // the counting sort: octant k's particles in [incl[k-1], incl[k]),
            // in reversed list order
            for (int i0 = i0w; i0 < i1w; i0 += 32) {
                const int i = i0 + lane;
                const bool in = i < i1w;
                const int o = in ? oct[i] : 8;
                const unsigned peers = __match_any_sync(0xFFFFFFFFu, o);
                int r = __popc(peers & lanemask_lt()), end_o = 0;
    #pragma unroll
                for (int k = 0; k < 8; ++k)
                    if (o == k) {
                        r += seen[k];
                        end_o = incl[k];
                    }
                if (in) {
                    tmp[end_o - 1 - r] = pis[bs + i];
                    tw[end_o - 1 - r] = wl[i];
                }
    #pragma unroll
                for (int k = 0; k < 8; ++k) seen[k] += __popc(__ballot_sync(0xFFFFFFFFu, in && o == k));
            }
            if (wide) {
                __syncthreads();
                for (int i = tid; i < nb; i += MB_THREADS) pis[bs + i] = tmp[i];
                __syncthreads();  // the first warp's next choice may read the list
                if (warp != 0) continue;
            } else {
                __syncwarp();
                for (int i = lane; i < nb; i += 32) pis[bs + i] = tmp[i];
                __syncwarp();
            }
            // the first warp: weights outside the FP32 range are summed exactly
            // now, in particle order as the reference sums them (octant k's
            // particles sit in [incl[k-1], incl[k]) in reversed particle order)
            double wo = 0.0;
            if (!approx) {
                int lo = 0, hi = 0;
    #pragma unroll
                for (int k = 0; k < 8; ++k)
                    if (lane == k) {
                        lo = incl[k] - cnt[k];
                        hi = incl[k];
                    }
                for (int j = hi - 1; j >= lo; --j) wo += tw[j];
            }
            // the children: lane k writes octant k's bin; the first non-empty
            // octant takes the parent's slot, the others are appended in
            // octant order
            int cl = 0, il = 0;
            float wfl = 0.f;
    #pragma unroll
            for (int k = 0; k < 8; ++k)
                if (lane == k) {
                    cl = cnt[k];
                    il = incl[k];
                    wfl = wf[k];
                }
            const unsigned nonempty = __ballot_sync(0xFFFFFFFFu, cl > 0);
            if (cl > 0) {
                const int kch = __popc(nonempty & lanemask_lt());
                const int id = kch == 0 ? bid : nbins + kch - 1;
                MergeBin b;
                for (int q = 0; q < 3; ++q) {
                    const bool upper = (lane >> q) & 1;
                    if (a.prm.bin_bounds_compute == BOUNDS_INHERIT) {
                        b.vmin[q] = upper ? mid[q] : P.vmin[q];
                        b.vmax[q] = upper ? P.vmax[q] : mid[q];
                    } else {
                        b.vmin[q] = P.vmin[q];
                        b.vmax[q] = P.vmax[q];
                    }
                }
                b.np = cl;
                b.w = approx ? -1.0 : wo;  // -1: the exact weight is still to be summed
                b.depth = P.depth + 1;
                b.start = bs + il - cl;
                b.end = bs + il - 1;
                b.refinable = (cl > 2) && (b.depth < a.prm.max_depth);
                b.pad = 0;
                s_wk[id] = b.refinable ? __double_as_longlong(approx ? (double)wfl : wo) : -1ll;
                bins[id] = b;
            }
    #pragma unroll
            for (int k = 0; k < 8; ++k) total += cnt[k] >= 2 ? 2 : cnt[k];
            total -= 2;
            nbins += nne - 1;
            more = nbins + 7 <= a.prm.max_Nbins;
            __syncwarp();
        }
        if (tid == 0) s_nbins = nbins;
        __syncthreads();
    }
    const int nbins = s_nbins;
    // the exact weights still missing: each bin's particles in particle order
    // (its range holds them reversed), one thread per bin
    for (int q = tid; q < nbins; q += MB_THREADS) {
        MergeBin& B = bins[q];
        if (B.w < 0.0) {
            double w = 0.0;
            for (int j = B.end; j >= B.start; --j) w += cv[pis[j]].w;
            B.w = w;
        }
    }
    __syncthreads();
    // the particles in list order (the octree scratch is dead: lx takes it)
    for (int i = tid; i < n; i += MB_THREADS) {
        const int q = pis[i];
        lv[i] = cv[q];
        lx[i] = A.pos[map_slot(p, q)];
    }
    __syncthreads();
    if (nbins == 1 && tid == 0) {
        double w = 0.0;
        for (int i = 0; i < n; ++i) w += lv[i].w;
        bins[0].w = w;
    }
    __syncthreads();

    // output position and rank among the bins of more than two particles of
    // every bin, in bin order: an exclusive scan over the bins (two per thread)
    int io[2] = {0, 0}, ib[2] = {0, 0};
    for (int q = 0; q < 2; ++q) {
        const int b = 2 * tid + q;
        if (b < nbins) {
            const MergeBin& B = bins[b];
            const int npe = B.w == 0.0 ? 0 : B.np;
            io[q] = npe >= 2 ? 2 : npe;
            ib[q] = npe > 2 ? 1 : 0;
        }
    }
    int so = io[0] + io[1], sb = ib[0] + ib[1];
    int xo = so, xb = sb;  // inclusive within the warp
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t1 = __shfl_up_sync(0xFFFFFFFFu, xo, o), t2 = __shfl_up_sync(0xFFFFFFFFu, xb, o);
        if (lane >= o) {
            xo += t1;
            xb += t2;
        }
    }
    if (lane == 31) {
        s_scan[warp][0] = xo;
        s_scan[warp][1] = xb;
    }
    __syncthreads();
    int wo0 = 0, wb0 = 0, tot_o = 0;
    for (int w = 0; w < NW; ++w) {
        if (w < warp) {
            wo0 += s_scan[w][0];
            wb0 += s_scan[w][1];
        }
        tot_o += s_scan[w][0];
    }
    {
        int po = wo0 + xo - so, pb = wb0 + xb - sb;
        for (int q = 0; q < 2; ++q) {
            const int b = 2 * tid + q;
            if (b < nbins) {
                s_pos[b] = po;
                s_kbig[b] = pb;
            }
            po += io[q];
            pb += ib[q];
        }
    }
    __syncthreads();

    // the bins a thread sums alone, largest first: a warp's FP64 work is set
    // by its largest bin, so bins of like size share a warp (counting sort by
    // particle count, descending; s_order reuses the scan's word arrays)
    __shared__ int s_hist[WIDE_BIN + 2];
    __shared__ int s_order[MB_BINS];
    for (int k = tid; k < WIDE_BIN + 2; k += MB_THREADS) s_hist[k] = 0;
    __syncthreads();
    for (int b = tid; b < nbins; b += MB_THREADS) {
        const MergeBin& B = bins[b];
        const int npe = B.w == 0.0 ? 0 : B.np;
        atomicAdd(&s_hist[npe > WIDE_BIN ? WIDE_BIN + 1 : npe], 1);
    }
    __syncthreads();
    if (tid == 0) {
        int run = 0;
        for (int k = WIDE_BIN + 1; k >= 0; --k) {
            const int t = s_hist[k];
            s_hist[k] = run;
            run += t;
        }
    }
    __syncthreads();
    for (int b = tid; b < nbins; b += MB_THREADS) {
        const MergeBin& B = bins[b];
        const int npe = B.w == 0.0 ? 0 : B.np;
        s_order[atomicAdd(&s_hist[npe > WIDE_BIN ? WIDE_BIN + 1 : npe], 1)] = b;
    }
    __syncthreads();

    // compute_bin_props! (:646-700) and compute_new_particles! (:736-933)
    Stream st;
    st.init(cell_seed(d, c), TAG_MERGE, (uint32_t)a.s, cell_step(d, c, a.step), cell_rid(d, c), 0);
    for (int r = tid; r < nbins; r += MB_THREADS) {
        const int b = s_order[r];
        const MergeBin B = bins[b];
        const int npe = B.w == 0.0 ? 0 : B.np;
        const int pos = s_pos[b];
        if (npe > 2 && npe <= WIDE_BIN) {
            double vm[3], xm[3], sv[3], sx[3];
            bin_moments_lane(lv, lx, B.start, B.end, 1.0 / B.w, vm, xm, sv, sx);
            emit_pair(a, st, s_kbig[b], B.w, vm, xm, sv, sx, ov + pos, ox + pos);
        } else if (npe >= 1 && npe <= 2) {
            for (int q = 0; q < npe; ++q) {
                ov[pos + q] = lv[B.start + q];
                ox[pos + q] = lx[B.start + q];
            }
        }
    }
    // bins of many particles: one warp each
    for (int b0 = 0; b0 < nbins; b0 += 32) {
        const int b = b0 + lane;
        bool wide = false;
        if (b < nbins) {
            const MergeBin& B = bins[b];
            wide = B.w != 0.0 && B.np > WIDE_BIN;
        }
        unsigned wmask = __ballot_sync(0xFFFFFFFFu, wide);
        for (int r = 0; wmask; ++r) {
            const int q = __ffs(wmask) - 1;
            wmask &= wmask - 1;
            if (r % NW != warp) continue;
            const MergeBin B = bins[b0 + q];
            double vm[3], xm[3], sv[3], sx[3];
            bin_moments_warp(lv, lx, B.start, B.end, 1.0 / B.w, vm, xm, sv, sx);
            if (lane == 0) {
                const int pos = s_pos[b0 + q];
                emit_pair(a, st, s_kbig[b0 + q], B.w, vm, xm, sv, sx, ov + pos, ox + pos);
            }
        }
    }
    __syncthreads();
    const int cur = tot_o;
    for (int j = tid; j < cur; j += MB_THREADS) {
        const int32_t slot = map_slot(p, j);
        A.wv[slot] = ov[j];
        A.pos[slot] = ox[j];
    }
    for (int j = cur + tid; j < n; j += MB_THREADS) {
        const int32_t slot = map_slot(p, j);
        A.wv[slot].w = 0.0;
        S.cell[slot] = -1;
    }
    if (tid == 0) {
        Indexer q = p;
        if (cur <= p.n1) {
            q.n1 = cur;
            q.n2 = 0;
            q.start2 = 0;
            if (cur == 0) q.start1 = 0;
        } else {
            q.n2 = cur - p.n1;
        }
        S.ind[c] = q;
        if (n > cur) atomicAdd((unsigned long long*)a.deleted, (unsigned long long)(n - cur));
        atomicAdd((unsigned long long*)a.merged, 1ull);
        atomicAdd(&d.counters->merges, 1ull);
    }
}

// Blocks take the next cell of up to MB_N particles from their own counter;
// larger cells are left to k_merge.
__global__ void __launch_bounds__(MB_THREADS, 1) k_merge_block(DomainView d, MergeArgs a, unsigned int* next)
{
    if (a.abort && *a.abort) return;
    if (a.step_ptr) a.step = *a.step_ptr;
    extern __shared__ __align__(16) char mb_smem[];
    __shared__ int s_cell;
    for (;;) {
        if (threadIdx.x == 0) {
            int c = a.ce;
            for (;;) {
                const int q = a.cb + (int)atomicAdd(next, 1u);
                if (q >= a.ce) break;
                const Indexer p = d.sp[a.s].ind[q];
                const int n = p.n1 + p.n2;
                if (n > 0 && n <= MB_N && (a.threshold < 0 || n > a.threshold)) {
                    c = q;
                    break;
                }
            }
            s_cell = c;
        }
        __syncthreads();
        const int c = s_cell;
        __syncthreads();
        if (c >= a.ce) break;
        merge_cell_block(d, a, c, mb_smem);
        __syncthreads();
    }
}

// largest particle count of the selected cells
__global__ void k_merge_sizes(DomainView d, int s, int cb, int ce, int64_t threshold, int64_t* out)
{
    int best = 0, cnt = 0;
    for (int c = cb + blockIdx.x * blockDim.x + threadIdx.x; c < ce; c += gridDim.x * blockDim.x) {
        const Indexer p = d.sp[s].ind[c];
        const int n = p.n1 + p.n2;
        if (n > 0 && (threshold < 0 || n > threshold)) {
            best = max(best, n);
            ++cnt;
        }
    }
    best = __reduce_max_sync(0xFFFFFFFFu, best);
    cnt = __reduce_add_sync(0xFFFFFFFFu, cnt);
    if ((threadIdx.x & 31) == 0) {
        atomicMax((unsigned long long*)out, (unsigned long long)best);
        atomicAdd((unsigned long long*)(out + 1), (unsigned long long)cnt);
    }
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// per-warp scratch layout for cells of up to nmax particles
void merge_layout(MergeArgs& a, int64_t nmax, int64_t target, int32_t max_Nbins)
{
    const int64_t outmax = std::max<int64_t>(target, 2);
    size_t off = align256((size_t)max_Nbins * sizeof(MergeBin));
    a.off_pis = off;
    off += align256(nmax * sizeof(int32_t));
    a.off_tmp = off;
    off += align256(nmax * sizeof(int32_t));
    a.off_w = off;
    off += align256(nmax * sizeof(double));
    a.off_tw = off;
    off += align256(nmax * sizeof(double));
    a.off_lv = off;
    off += align256(nmax * sizeof(PV));
    a.off_lx = off;
    off += align256(nmax * sizeof(PX));
    a.off_oct = off;
    off += align256(nmax);
    a.off_ov = off;
    off += align256(outmax * sizeof(PV));
    a.off_ox = off;
    off += align256(outmax * sizeof(PX));
    a.stride = off;
    a.nmax = (int32_t)nmax;
}

void check_octree(const mz_octree_params* prm, int64_t target)
{
    MZ_REQUIRE(prm->split == 1, "mz_merge_octree_n2: only OctreeBinMidSplit (split = 1) is implemented");
    MZ_REQUIRE(prm->init_bin_bounds >= 1 && prm->init_bin_bounds <= 3, "mz_merge_octree_n2: bad init_bin_bounds");
    MZ_REQUIRE(prm->bin_bounds_compute == 1 || prm->bin_bounds_compute == 2,
               "mz_merge_octree_n2: bad bin_bounds_compute");
    MZ_REQUIRE(prm->max_Nbins >= 8, "mz_merge_octree_n2: max_Nbins must be at least 8 (one split)");
    MZ_REQUIRE(target <= (1 << 30), "mz_merge_octree_n2: target_np too large");
}

void ensure_merge_scratch(mz_domain* d, size_t need)
{
    if (need <= d->merge_scratch_bytes) return;
    cudaFree(d->d_merge_scratch);
    d->d_merge_scratch = nullptr;
    d->merge_scratch_bytes = 0;
    MZ_CK(cudaMalloc(&d->d_merge_scratch, need));
    d->merge_scratch_bytes = need;
}

}  // namespace

namespace {
// the block form takes the cells it can hold when the target fits its bins
bool merge_block_usable(int64_t target) { return target <= MB_BINS; }

// blocks of the block form that fit the GPU at once; the first call on a
// device (made before any stream capture: merge_fused_reserve, launch_merge)
// raises the kernel's shared-memory limit
int merge_block_grid(mz_domain* d)
{
    static int grid[64] = {0};
    const int dev = d->ctx->device;
    if (dev >= 0 && dev < 64 && grid[dev] > 0) return grid[dev];
    MZ_CK(cudaFuncSetAttribute(k_merge_block, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)MB_SMEM));
    int per_sm = 0;
    MZ_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_merge_block, MB_THREADS, MB_SMEM));
    MZ_REQUIRE(per_sm >= 1, "merge: the block form does not fit on an SM");
    const int g = d->ctx->num_sms * per_sm;
    if (dev >= 0 && dev < 64) grid[dev] = g;
    return g;
}
}  // namespace

int merge_fused_warps(mz_domain* d) { return d->ctx->num_sms * 2; }

void merge_fused_reserve(mz_domain* d, int64_t nmax, int64_t target, const mz_octree_params* prm)
{
    check_octree(prm, target);
    MergeArgs a;
    memset(&a, 0, sizeof a);
    merge_layout(a, nmax, target, prm->max_Nbins);
    ensure_merge_scratch(d, (size_t)merge_fused_warps(d) * a.stride);
    if (merge_block_usable(target)) merge_block_grid(d);
}


void launch_merge_fused(mz_domain* d, int s, int64_t threshold, int64_t target, const mz_octree_params* prm,
                        const mz_grid1d* g, const uint32_t* step_ptr, const int* abort, int64_t nmax,
                        long long* words3)
{
    mz_ctx* c = d->ctx;
    MergeArgs a;
    memset(&a, 0, sizeof a);
    a.s = s;
    a.cb = 0;
    a.ce = (int)d->n_cells;
    a.threshold = threshold;
    a.target = (int32_t)target;
    a.prm = *prm;
    a.clamp = g != nullptr;
    if (g) {
        a.min_x = g->min_x;
        a.max_x = g->max_x;
    }
    merge_layout(a, nmax, target, prm->max_Nbins);
    const int warps = merge_fused_warps(d);
    MZ_REQUIRE((size_t)warps * a.stride <= d->merge_scratch_bytes, "merge: scratch not reserved");
    a.scratch = static_cast<char*>(d->d_merge_scratch);
    a.deleted = reinterpret_cast<int64_t*>(words3);
    a.merged = reinterpret_cast<int64_t*>(words3 + 1);
    a.next = reinterpret_cast<unsigned int*>(words3 + 2);
    a.step_ptr = step_ptr;
    a.abort = abort;
    DomainView v = make_view(d);
    MZ_CK(cudaMemsetAsync(a.next, 0, 2 * sizeof(long long), c->stream));
    if (merge_block_usable(target)) {
        // cells of up to MB_N particles in the block form, the rest by warps
        MZ_LAUNCH(c, "merge_block", k_merge_block, merge_block_grid(d), MB_THREADS, MB_SMEM, v, a,
                  reinterpret_cast<unsigned int*>(words3 + 3));
        a.min_n = MB_N;
    }
    MZ_LAUNCH(c, "merge", k_merge, warps, 32, 0, v, a);
}

void launch_merge(mz_domain* d, int s, int64_t cb, int64_t ce, int64_t threshold, int64_t target,
                  const mz_octree_params* prm, const mz_grid1d* g, uint64_t step, int64_t* n_merged)
{
    mz_ctx* c = d->ctx;
    check_octree(prm, target);
    if (n_merged) *n_merged = 0;
    if (ce <= cb) return;
    DomainView v = make_view(d);
    // sizes of the selected cells decide the scratch per warp
    MZ_CK(cudaMemsetAsync(d->d_scalar, 0, 4 * sizeof(int64_t), c->stream));
    const int sb = (int)std::max<int64_t>(1, std::min<int64_t>(div_up(ce - cb, 256), (int64_t)c->num_sms * 4));
    MZ_LAUNCH(c, "merge_sizes", k_merge_sizes, sb, 256, 0, v, s, (int)cb, (int)ce, threshold, d->d_scalar);
    MZ_CK(cudaMemcpyAsync(d->h_scalar, d->d_scalar, 2 * sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
    MZ_CK(cudaStreamSynchronize(c->stream));
    const int64_t nmax = d->h_scalar[0], ncells = d->h_scalar[1];
    if (ncells == 0) return;

    MergeArgs a;
    memset(&a, 0, sizeof a);
    a.s = s;
    a.cb = (int)cb;
    a.ce = (int)ce;
    a.threshold = threshold;
    a.target = (int32_t)target;
    a.prm = *prm;
    a.clamp = g != nullptr;
    if (g) {
        a.min_x = g->min_x;
        a.max_x = g->max_x;
    }
    a.step = (uint32_t)step;
    merge_layout(a, nmax, target, prm->max_Nbins);
    // one warp per block: the merging warps spread over all SMs (a merge is a
    // long sequential chain; SMs shared by several merging warps slow each)
    const int warps_wanted = (int)std::min<int64_t>(ncells, (int64_t)c->num_sms * 16);
    const int blocks = std::max(1, warps_wanted);
    ensure_merge_scratch(d, (size_t)blocks * a.stride);
    a.scratch = static_cast<char*>(d->d_merge_scratch);
    a.deleted = d->d_scalar + 2;
    a.merged = d->d_scalar + 3;
    a.next = reinterpret_cast<unsigned int*>(d->d_scalar + 8);
    MZ_CK(cudaMemsetAsync(d->d_scalar + 8, 0, 2 * sizeof(int64_t), c->stream));
    bool warps_needed = true;
    if (merge_block_usable(target)) {
        // cells of up to MB_N particles in the block form, the rest by warps
        const int bgrid = (int)std::min<int64_t>(ncells, (int64_t)merge_block_grid(d));
        MZ_LAUNCH(c, "merge_block", k_merge_block, bgrid, MB_THREADS, MB_SMEM, v, a,
                  reinterpret_cast<unsigned int*>(d->d_scalar + 9));
        a.min_n = MB_N;
        warps_needed = nmax > MB_N;
    }
    if (warps_needed) MZ_LAUNCH(c, "merge", k_merge, blocks, 32, 0, v, a);
    MZ_CK(cudaMemcpyAsync(d->h_scalar + 2, d->d_scalar + 2, 2 * sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
    MZ_CK(cudaStreamSynchronize(c->stream));
    SpeciesHost& S = d->sp[s];
    const int64_t deleted = d->h_scalar[2];
    S.n_total -= deleted;
    if (deleted > 0) S.compact = false;
    if (n_merged) *n_merged = d->h_scalar[3];
}
