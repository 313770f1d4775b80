// NTC of one large cell by a whole block: the block-per-cell mapping of the
// equal-weight candidate loop (ntc_equal_weight!, collision_ntc.jl:479-521 and
// :554-595).
//
// ntc_cell evaluates at most G <= 32 candidates of a cell at a time; a cell of
// N particles offers about sqrt(pi N / 8) conflict-free candidates, so cells of
// thousands of particles leave most of that parallelism unused and their
// sequential chain of batches sets the length of a step.  Here a block of
// NTC_BLOCK threads evaluates up to NTC_BLOCK candidates per batch with the
// same semantics:
//   * the batch ends before the first candidate that touches a particle of an
//     earlier candidate in the batch: every particle of the batch goes into a
//     shared-memory hash table that keeps the smallest candidate index using
//     it (open addressing, at most 2 NTC_BLOCK keys in NTC_TABLE slots);
//   * an inclusive block max-scan of sigma*g*w bit patterns gives every
//     candidate the exact running maximum;
//   * draws, screening, acceptance and scattering are those of ntc_cell, so
//     the result equals the sequential loop (and ntc_cell) bit for bit.
// A warp-wide FP64 instruction holds the SM's FP64 pipe for 16 clocks however
// few of its lanes are active, and one block is the only FP64 user of its cell.
// The two long FP64 sequences therefore run on compacted threads: the exact
// sigma*g*w (pow, about 1 % of the candidates) and the scattering of the
// accepted candidates (about a third) are listed in shared memory and done by
// the first threads of the block, each resuming the candidate's own stream at
// the draw it had reached.
#pragma once

#include <climits>

#include "cell_ops.cuh"

namespace mz {

constexpr int NTC_BLOCK = 256;
constexpr int NTC_TABLE = 2048;  // power of two, > 2 NTC_BLOCK / 0.5

struct NtcBlockShared {
    int32_t key[NTC_TABLE];
    int32_t first[NTC_TABLE];
    long long wmax[NTC_BLOCK / 32];
    int32_t end;
    int32_t accepted;
    int32_t n_exact;
    long long last_max;
    // per candidate of the batch (indexed by its thread), for the compacted work
    int32_t list[NTC_BLOCK];   // candidates needing the exact sigma*g*w, then the accepted ones
    int32_t slot1[NTC_BLOCK], slot2[NTC_BLOCK];
    uint32_t draws[NTC_BLOCK];  // draws taken from the candidate's stream before scattering
    double g2[NTC_BLOCK];
    double val[NTC_BLOCK];      // the pair's larger weight, then its exact sigma*g*w
};

__device__ __forceinline__ uint32_t ntc_hash(int32_t t) { return ((uint32_t)t * 0x9E3779B1u) >> (32 - 11); }

__device__ __forceinline__ void ntc_table_insert(NtcBlockShared& sh, int32_t t, int32_t cand)
{
    uint32_t h = ntc_hash(t);
    for (int probe = 0; probe < NTC_TABLE; ++probe) {
        const int32_t prev = atomicCAS(&sh.key[h], -1, t);
        if (prev == -1 || prev == t) {
            atomicMin(&sh.first[h], cand);
            return;
        }
        h = (h + 1) & (NTC_TABLE - 1);
    }
}

__device__ __forceinline__ int32_t ntc_table_first(const NtcBlockShared& sh, int32_t t)
{
    uint32_t h = ntc_hash(t);
    for (int probe = 0; probe < NTC_TABLE; ++probe) {
        if (sh.key[h] == t) return sh.first[h];
        h = (h + 1) & (NTC_TABLE - 1);
    }
    return INT_MAX;
}

// Equal-weight candidate loop of one cell by the whole block (all threads call
// it with identical arguments).  Returns the new running maximum and the
// number of accepted collisions (valid in every thread).
//
// A batch's index draws and conflict detection depend only on where the batch
// starts, so they run one batch ahead: while the block loads, screens, tests
// and scatters batch b, it also draws the candidates of batch b+1 (which
// starts where b ends), fills the conflict table with them and finds their
// first conflict, in the same barrier-separated steps.  A batch then costs
// five block barriers, and the Philox work overlaps the particle loads.
//   step 1: b's loads, g^2, screening, exact list  | b+1's draws, table clear
//   step 2: b's exact sigma*g*w (compacted)        | b+1's table inserts
//   step 3: b's per-warp max-scan                  | b+1's first conflict
//   step 4: b's scan across warps, acceptance, accepted list
//   step 5: b's scattering (compacted); b+1's length is final
__device__ __forceinline__ NtcResult ntc_cell_block(NtcBlockShared& sh, const Interaction& I, bool single,
                                                    int32_t ncoll, double smax, const Cols& P1, const Cols& P2,
                                                    const Indexer& p1, const Indexer& p2, const double2* trig,
                                                    uint64_t seed, uint32_t pc, uint32_t stp, uint32_t rid)
{
    const int tid = threadIdx.x;
    const int lane = tid & 31, wid = tid >> 5;
    const double vexp = fma(-2.0, I.vhs_o, 1.0);
    const float lC = I.vhs_factor > 0.0 ? log2_pos(I.vhs_factor) : 1e30f;
    const bool screen = fabsf(lC) < LOG_RANGE;
    const float ex = 1.0f - (float)I.vhs_o;
    const int32_t nl1 = p1.n1 + p1.n2;
    const int32_t nl2 = single ? nl1 : p2.n1 + p2.n2;
    const int32_t tagk = single ? 0 : (int32_t)0x40000000;  // species 2 particles get their own keys
    NtcResult R;
    R.perf = R.eqw = R.nsp1 = R.nsp2 = 0;
    R.smax = smax;
    if (ncoll <= 0) return R;

    // candidate jn + tid of the batch starting at jn: its index draws, and
    // (whole block) the cleared conflict table and the batch's maximum length
    auto draw = [&](int32_t jn, Stream& st, int32_t& i, int32_t& k) -> bool {
        const int32_t j = jn + tid;
        const bool valid = j < ncoll;
        st.init(seed, TAG_CAND, pc, stp, rid, (uint32_t)j);
        i = -1;
        k = -1;
        if (valid) {
            i = floor_u52_times(st.u52(), nl1);
            k = floor_u52_times(st.u52(), nl2);
            if (single) {
                int guard = 0;
                while (i == k && guard++ < (1 << 20)) k = floor_u52_times(st.u52(), nl1);
            }
        }
        for (int q = tid; q < NTC_TABLE; q += NTC_BLOCK) {
            sh.key[q] = -1;
            sh.first[q] = INT_MAX;
        }
        if (tid == 0) sh.end = max(0, min(NTC_BLOCK, ncoll - jn));
        return valid;
    };
    auto insert = [&](bool valid, int32_t i, int32_t k) {
        if (valid) {
            ntc_table_insert(sh, i, tid);
            ntc_table_insert(sh, k | tagk, tid);
        }
    };
    // the batch ends before the first candidate that touches a particle of an
    // earlier candidate in the batch
    auto first_conflict = [&](bool valid, int32_t i, int32_t k) {
        const bool conflict = valid && (ntc_table_first(sh, i) < tid || ntc_table_first(sh, k | tagk) < tid);
        const int cmin = __reduce_min_sync(0xFFFFFFFFu, conflict ? tid : INT_MAX);
        if (lane == 0 && cmin != INT_MAX) atomicMin(&sh.end, cmin);
    };

    // batch 0's draws and length
    Stream st;
    int32_t i, k;
    if (tid == 0) sh.n_exact = 0;
    {
        const bool valid = draw(0, st, i, k);
        __syncthreads();
        insert(valid, i, k);
        __syncthreads();
        first_conflict(valid, i, k);
        __syncthreads();
    }
    int B = sh.end;
    __syncthreads();  // every thread has read sh.end before step 1 rewrites it
    for (int32_t j0 = 0; j0 < ncoll;) {  // j0 and B are the same in every thread
        const int32_t jn = j0 + B;
        const bool act = tid < B;
        // ---- step 1
        if (tid == 0) sh.accepted = 0;
        const float l_smax = log2_pos(smax);
        const bool screen_b = screen && fabsf(l_smax) < 2.0f * LOG_RANGE;
        int32_t si = 0, sk = 0;
        double g2 = 0.0, g = 0.0, sgw = -1.0, wmax = 0.0;
        bool has = false, exact = false, have_g = false;
        float ls = 0.0f;
        if (act) {
            si = map_slot(p1, i);
            sk = map_slot(p2, k);
            const PV a = P1.wv[si];
            const PV b = P2.wv[sk];
            const double gx = a.vx - b.vx, gy = a.vy - b.vy, gz = a.vz - b.vz;
            g2 = (gx * gx + gy * gy) + gz * gz;
            wmax = dmax_pos(a.w, b.w);
            if ((uint64_t)__double_as_longlong(g2) > G2_TINY_BITS) {
                has = true;
            } else {
                g = sqrt(g2);
                have_g = true;
                has = g > EPS;
            }
            if (has) {
                const float lw = log2_pos(wmax), lg = log2_pos(g2);
                ls = lC + lw + ex * lg;
                exact = !screen_b || fabsf(lw) >= LOG_RANGE || fabsf(lg) >= LOG_RANGE ||
                        ls > l_smax - SCREEN_MARGIN;
            }
            sh.g2[tid] = g2;
            if (exact) {
                sh.val[tid] = wmax;
                sh.list[atomicAdd(&sh.n_exact, 1)] = tid;
            }
        }
        Stream sn;
        int32_t ni, nk;
        const bool nvalid = draw(jn, sn, ni, nk);
        __syncthreads();
        // ---- step 2: exact sigma*g*w on compacted threads (each value
        // depends on its own candidate only)
        const int ne = sh.n_exact;
        for (int q = tid; q < ne; q += NTC_BLOCK) {
            const int t = sh.list[q];
            const double gt = sqrt(sh.g2[t]);
            sh.val[t] = I.vhs_factor * pow(gt, vexp) * gt * sh.val[t];
        }
        insert(nvalid, ni, nk);
        __syncthreads();
        // ---- step 3: inclusive max-scan of the sigma*g*w bit patterns, per warp
        if (act && exact) sgw = sh.val[tid];
        long long mk = max_key(sgw, act && exact);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long t = __shfl_up_sync(0xFFFFFFFFu, mk, o);
            if (lane >= o) mk = max(mk, t);
        }
        if (lane == 31) sh.wmax[wid] = mk;
        first_conflict(nvalid, ni, nk);
        __syncthreads();
        // ---- step 4: the scan across warps and the acceptance tests
        if (tid == 0) sh.n_exact = 0;
        long long before = __double_as_longlong(smax);
        for (int w = 0; w < wid; ++w) before = max(before, sh.wmax[w]);
        mk = max(mk, before);
        if (tid == B - 1) sh.last_max = mk;
        const double m = __longlong_as_double(mk);
        bool acc = false;
        if (act && has) {
            const uint64_t um = st.u52();
            if (exact) {
                acc = u52_to_double(um) < sgw / m;
            } else {
                const float lm = log2_pos(m);
                const float dl = ls - lm - log2_u52(um);
                if (dl > SCREEN_MARGIN && fabsf(lm) < 2.0f * LOG_RANGE) {
                    acc = true;
                } else if (dl >= -SCREEN_MARGIN || fabsf(lm) >= 2.0f * LOG_RANGE) {
                    if (!have_g) g = sqrt(g2);
                    have_g = true;
                    const double se = I.vhs_factor * pow(g, vexp) * g * wmax;
                    acc = u52_to_double(um) < se / m;
                }
            }
        }
        if (acc) {
            sh.slot1[tid] = si;
            sh.slot2[tid] = sk;
            sh.draws[tid] = st.n;
            sh.list[atomicAdd(&sh.accepted, 1)] = tid;
        }
        __syncthreads();
        // ---- step 5: scatter_vhs! of the accepted candidates on compacted
        // threads; the batch's candidates share no particle, so the order is free
        const int na = sh.accepted;
        const int Bn = sh.end;
        R.perf += na;
        smax = __longlong_as_double(sh.last_max);
        for (int q = tid; q < na; q += NTC_BLOCK) {
            const int t = sh.list[q];
            Stream sc;
            sc.init(seed, TAG_CAND, pc, stp, rid, (uint32_t)(j0 + t));
            sc.n = sh.draws[t];
            const int32_t ti = sh.slot1[t], tk = sh.slot2[t];
            const PV ta = P1.wv[ti], tb = P2.wv[tk];
            const double gt = sqrt(sh.g2[t]);
            const double cx = I.mu1 * ta.vx + I.mu2 * tb.vx;
            const double cy = I.mu1 * ta.vy + I.mu2 * tb.vy;
            const double cz = I.mu1 * ta.vz + I.mu2 * tb.vz;
            double sphi, cphi;
            sincos_2pi_u52(trig, sc.u52(), sphi, cphi);
            const double ct = fma(2.0, sc.uniform(), -1.0);
            const double sth = sqrt(1.0 - ct * ct);
            const double nx = gt * (sth * cphi), ny = gt * (sth * sphi), nz = gt * ct;
            P1.wv[ti] = PV{ta.w, cx + I.mu2 * nx, cy + I.mu2 * ny, cz + I.mu2 * nz};
            P2.wv[tk] = PV{tb.w, cx - I.mu1 * nx, cy - I.mu1 * ny, cz - I.mu1 * nz};
        }
        // the next batch reads the scattered velocities; the shared counters
        // and lists are rewritten from here on
        __syncthreads();
        j0 = jn;
        B = Bn;
        st = sn;
        i = ni;
        k = nk;
    }
    R.eqw = R.perf;
    R.smax = smax;
    return R;
}

}  // namespace mz
