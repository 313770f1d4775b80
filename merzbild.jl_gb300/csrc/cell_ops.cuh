// Per-cell device routines shared by the standalone kernels (ntc.cu,
// props.cu, convect.cu) and the fused step kernel (step.cu), so both paths
// execute the same arithmetic.
#pragma once

#include "mz_internal.cuh"

namespace mz {

// ------------------------------------------------------------------ NTC
// compute_n_coll_single_species / _two_species (collision_ntc.jl:173-197);
// also resets the per-call counters like ntc! does (:351-353).
__device__ __forceinline__ int32_t ntc_ncoll(const DomainView& d, CollisionFactors& cf, bool single, int64_t n1,
                                             int64_t n2, double dt, double V, uint64_t seed, uint32_t pc, uint32_t stp,
                                             uint32_t rid)
{
    Stream st;
    st.init(seed, TAG_NCOLL, pc, stp, rid, 0);
    const double U = st.uniform();
    double f;
    if (single)
        f = 0.5 * dt * (double)n1 * (double)(n1 - 1) * cf.smax / V + U;
    else
        f = dt * (double)n1 * (double)n2 * cf.smax / V + U;
    double fl = floor(f);
    if (!(fl < 1.0e9)) {
        set_status(d, ST_CAPACITY);
        fl = fl != fl ? 0.0 : 1.0e9;
    }
    const int32_t nci = (int32_t)fl;
    cf.n1 = (int32_t)n1;
    cf.n2 = (int32_t)(single ? n1 : n2);
    cf.n_coll = nci;
    cf.n_coll_performed = 0;
    cf.n_eq_w_coll_performed = 0;
    cf.n_split = 0;
    return nci;
}


struct NtcResult {
    double smax;
    int32_t perf, eqw, nsp1, nsp2;
};

// Screening of sigma*g*w_max in the FP32 log domain.  The FP64 pipe of GB300
// runs at ~1/60 of the FP32 rate, and FP64 pow and division dominate a
// candidate's cost.  log2(s) = log2(C) + log2(w_max) + (1 - omega) log2(g^2) is
// formed from FP32 approximations; the exact FP64 value is computed only where
// it can change a decision:
//   * a candidate whose s may reach the running maximum (it may raise it), and
//   * an acceptance test U < s / max whose two sides lie within SCREEN_MARGIN.
// Error budget: every log2 term is kept below LOG_RANGE in magnitude (terms
// beyond it take the exact path), so each of the <= 7 FP32 additions and
// products rounds by at most 2^-14, and each approximate log2 errs by < 1e-6;
// the total stays below 5e-4 < SCREEN_MARGIN.  Every decision taken on the
// screened value is therefore the decision of the all-FP64 loop, and so is
// the running maximum (screened candidates lie strictly below it).
// Weights are positive, so max(w_i, w_k) may compare bit patterns.
constexpr float SCREEN_MARGIN = 1e-3f;                    // log2 units
constexpr float LOG_RANGE = 128.0f;                       // |log2| bound of a screened term
constexpr uint64_t G2_TINY_BITS = 0x3990000000000000ull;  // bits of 4 eps^2 = 2^-102

__device__ __forceinline__ double dmax_pos(double a, double b)
{   // max of two positive doubles through their bit patterns
    const long long x = __double_as_longlong(a), y = __double_as_longlong(b);
    return __longlong_as_double(x > y ? x : y);
}

// Bit pattern of sigma*g*w for the running-maximum scan: positive doubles
// order like their bit patterns; "no value" and NaN (which never raise the
// maximum: `smax < s` is false) map to -1.
__device__ __forceinline__ long long max_key(double s, bool present)
{
    const long long k = __double_as_longlong(s);
    return (present && k <= 0x7FF0000000000000ll) ? k : -1ll;
}

// The candidate loop of ntc! / ntc_equal_weight! for one cell, executed by
// one group of G lanes (all G lanes call it with identical arguments; a warp
// holds 32 / G groups, each on its own cell).
//   P1, P2: particle columns of the two species (same for single species)
//   p1, p2: the cell's indexers; grown in place by splits
//   cell1/key1, cell2/key2: slot-owner arrays, written for split particles
//   b1/b2: first reserved slot for split particles of species 1/2
// Candidates are evaluated in conflict-free batches of up to G (see ntc.cu).
// A warp instruction serves every group, so with G = 8 one FP64 instruction
// covers the candidates of four cells instead of the ~12 conflict-free
// candidates one cell offers.
template <bool EQW, int G>
__device__ __forceinline__ NtcResult ntc_cell(const DomainView& d, const Interaction& I, bool single, int c,
                                              int32_t ncoll, double smax, const Cols& P1, const Cols& P2,
                                              Indexer& p1, Indexer& p2, int32_t* cell1, int32_t* key1,
                                              int32_t* cell2, int32_t* key2, int32_t b1, int32_t b2, double dw_tol,
                                              uint64_t seed, uint32_t pc, uint32_t stp, uint32_t rid)
{
    const WarpGroup<G> grp;
    const int gl = grp.rank;
    const double vexp = fma(-2.0, I.vhs_o, 1.0);  // sigma_vhs exponent, collision_cross_sections.jl:179-181
    const float lC = I.vhs_factor > 0.0 ? log2_pos(I.vhs_factor) : 1e30f;
    const bool screen = fabsf(lC) < LOG_RANGE;
    const float ex = 1.0f - (float)I.vhs_o;       // s = C w_max (g^2)^(1 - omega)
    NtcResult R;
    R.perf = 0;
    R.eqw = 0;
    R.nsp1 = 0;
    R.nsp2 = 0;
    for (int32_t j0 = 0; j0 < ncoll;) {
        const int32_t j = j0 + gl;
        const bool valid = j < ncoll;
        Stream st;
        st.init(seed, TAG_CAND, pc, stp, rid, (uint32_t)j);
        int32_t i = -1, k = -2;
        if (valid) {
            // i, k = floor(rand() * n_local) (collision_ntc.jl:358-363)
            const int32_t nl1 = p1.n1 + p1.n2;
            const int32_t nl2 = single ? nl1 : p2.n1 + p2.n2;
            i = floor_u52_times(st.u52(), nl1);
            k = floor_u52_times(st.u52(), nl2);
            if (single) {
                int guard = 0;
                while (i == k && guard++ < (1 << 20)) k = floor_u52_times(st.u52(), nl1);
            }
        }
        // the batch ends before the first candidate that touches a particle
        // of an earlier candidate in the batch
        bool conflict = false;
#pragma unroll
        for (int src = 0; src < G - 1; ++src) {
            const int32_t ii = grp.shfl(i, src);
            const int32_t kk = grp.shfl(k, src);
            if (src < gl) {
                if (single)
                    conflict |= (ii == i) | (ii == k) | (kk == i) | (kk == k);
                else
                    conflict |= (ii == i) | (kk == k);
            }
        }
        const unsigned cm = grp.ballot(valid && conflict);
        const int nvalid = min(G, ncoll - j0);
        int B = cm ? min(nvalid, __ffs(cm) - 1) : nvalid;
        bool act = gl < B;

        const float l_smax = log2_pos(smax);
        const bool screen_b = screen && fabsf(l_smax) < 2.0f * LOG_RANGE;
        int32_t si = 0, sk = 0;
        PV a, b;
        a.w = b.w = 0.0;
        double g2 = 0.0, g = 0.0, sgw = -1.0, wmax = 0.0;
        bool has = false, exact = false, have_g = false;
        float ls = 0.0f;
        if (act) {
            si = map_slot(p1, i);
            sk = map_slot(p2, k);
            a = P1.wv[si];
            b = P2.wv[sk];
            // compute_g! (collision_utils.jl:388-391)
            const double gx = a.vx - b.vx, gy = a.vy - b.vy, gz = a.vz - b.vz;
            g2 = (gx * gx + gy * gy) + gz * gz;
            wmax = dmax_pos(a.w, b.w);
            // g > eps() (collision_ntc.jl:375) is certain unless g^2 <= 4 eps^2
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
                if (exact) {
                    if (!have_g) g = sqrt(g2);
                    have_g = true;
                    sgw = I.vhs_factor * pow(g, vexp) * g * wmax;  // sigma_vhs(g) * g * max(w_i, w_k)
                }
            }
        }
        // running (sigma g w)_max each candidate is tested against
        // (collision_ntc.jl:229), as an inclusive max-scan over the batch on
        // bit patterns; candidates screened out lie below smax
        long long mk = max_key(sgw, act && exact);
#pragma unroll
        for (int o = 1; o < G; o <<= 1) {
            const long long t = grp.up(mk, o);
            if (gl >= o) mk = max(mk, t);
        }
        mk = max(mk, __double_as_longlong(smax));
        const double m = __longlong_as_double(mk);
        bool acc = false;
        if (act && has) {
            // rand() < sigma_g_w / (sigma g w)_max (collision_ntc.jl:231)
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
        bool spl = false;
        if (!EQW) {
            spl = acc && !(fabs(a.w - b.w) < dw_tol);
            const unsigned sm = grp.ballot(spl);
            if (sm) B = min(B, __ffs(sm));  // the batch ends after the first split
        }
        act = gl < B;
        acc = acc && act;
        spl = spl && act;
        int side = 0;
        if (acc) {
            double wi = a.w, wk = b.w;  // weights after a split
            if (!have_g) g = sqrt(g2);
            // compute_com! (collision_utils.jl:374-376)
            const double cx = I.mu1 * a.vx + I.mu2 * b.vx;
            const double cy = I.mu1 * a.vy + I.mu2 * b.vy;
            const double cz = I.mu1 * a.vz + I.mu2 * b.vz;
            if (!EQW && spl) {
                // split the heavier particle; the new particle keeps the
                // pre-collision velocity and position (collision_ntc.jl:235-267)
                const bool heavy_i = a.w > b.w;
                side = heavy_i ? 1 : 2;
                const Cols& PP = heavy_i ? P1 : P2;
                const int32_t src = heavy_i ? si : sk;
                const PV& h = heavy_i ? a : b;
                const double wl = heavy_i ? b.w : a.w;
                int32_t ns_;
                if (heavy_i || single)
                    ns_ = b1 + R.nsp1;
                else
                    ns_ = b2 + R.nsp2;
                PP.wv[ns_] = PV{h.w - wl, h.vx, h.vy, h.vz};
                PP.pos[ns_] = PP.pos[src];
                int32_t* cl = (heavy_i || single) ? cell1 : cell2;
                int32_t* ky = (heavy_i || single) ? key1 : key2;
                cl[ns_] = c;
                ky[ns_] = c;
                if (heavy_i)
                    wi = wl;
                else
                    wk = wl;
            }
            // scatter_vhs! (collision_scattering.jl:17-29): phi = 2 pi rand(),
            // cos(theta) = 2 rand() - 1
            double sphi, cphi;
            sincos_2pi_u52(d.trig, st.u52(), sphi, cphi);
            const double ct = fma(2.0, st.uniform(), -1.0);
            const double sth = sqrt(1.0 - ct * ct);
            const double nx = g * (sth * cphi), ny = g * (sth * sphi), nz = g * ct;
            P1.wv[si] = PV{wi, cx + I.mu2 * nx, cy + I.mu2 * ny, cz + I.mu2 * nz};
            P2.wv[sk] = PV{wk, cx - I.mu1 * nx, cy - I.mu1 * ny, cz - I.mu1 * nz};
        }
        const unsigned am = grp.ballot(acc);
        R.perf += __popc(am);
        if (EQW)
            R.eqw += __popc(am);
        else
            R.eqw += __popc(grp.ballot(acc && fabs(a.w - b.w) < dw_tol));
        smax = __longlong_as_double(grp.shfl(mk, B - 1));
        if (!EQW) {
            const int sd = grp.shfl(side, B - 1);
            if (sd == 1 || (sd == 2 && single)) {
                if (p1.n2 == 0) p1.start2 = b1;
                p1.n2 += 1;
                R.nsp1 += 1;
                if (single) p2 = p1;
            } else if (sd == 2) {
                if (p2.n2 == 0) p2.start2 = b2;
                p2.n2 += 1;
                R.nsp2 += 1;
            }
        }
        grp.sync();
        j0 += B;
    }
    R.smax = smax;
    return R;
}

// ntc! with splitting (collision_ntc.jl:223-270) for one single-species cell,
// one group of G lanes, with batches that run through several splits.
//
// In ntc_cell a batch ends at its first split, because the split appends a
// particle and every later candidate draws its indices from the new count:
// i = floor(rand() * n_local).  Here each lane evaluates its candidate for V
// counts at once, n_local + v for v = 0 .. V-1 (its draws do not depend on
// the count, only their scaling does), and the batch is then resolved in
// candidate order, segment by segment: the lanes after the v-th split of the
// batch take their version v values.  Within the batch the sequential loop is
// reproduced exactly:
//   * the running (sigma g w)_max is an inclusive max-scan over the resolved
//     versions, so every acceptance test sees the maximum the loop would;
//   * a candidate that touches a particle an earlier accepted candidate of
//     the batch changed, or a particle a split of the batch created, ends the
//     batch before it (rejected candidates change nothing, so only accepted
//     ones count);
//   * the batch ends after its V-th split.
// All accepted candidates of a batch then collide at once, on disjoint
// particles.  The position of a split-off particle (its parent's, unchanged
// by collisions) is copied after the cell's loop; until then its key entry
// holds the parent's slot.  (The chain of keys only leads back: a parent
// split off in this call has a smaller slot than its children.)
constexpr int NTC_SPLIT_VERSIONS = 3;

template <int G, int V>
__device__ __forceinline__ NtcResult ntc_cell_split(const DomainView& d, const Interaction& I, int c, int32_t ncoll,
                                                    double smax, const Cols& P, Indexer& p, int32_t* cell,
                                                    int32_t* key, int32_t b1, double dw_tol, uint64_t seed,
                                                    uint32_t pc, uint32_t stp, uint32_t rid)
{
    const WarpGroup<G> grp;
    const int gl = grp.rank;
    const double vexp = fma(-2.0, I.vhs_o, 1.0);  // sigma_vhs exponent, collision_cross_sections.jl:179-181
    const float lC = I.vhs_factor > 0.0 ? log2_pos(I.vhs_factor) : 1e30f;
    const bool screen = fabsf(lC) < LOG_RANGE;
    const float ex = 1.0f - (float)I.vhs_o;
    NtcResult R;
    R.perf = 0;
    R.eqw = 0;
    R.nsp1 = 0;
    R.nsp2 = 0;
    for (int32_t j0 = 0; j0 < ncoll;) {
        const int32_t j = j0 + gl;
        const bool valid = j < ncoll;
        const int nvalid = min(G, ncoll - j0);
        Stream st;
        st.init(seed, TAG_CAND, pc, stp, rid, (uint32_t)j);
        // the candidate's first six draws: i, k, then (k redrawn while equal
        // to i) the acceptance draw and the two scattering draws
        uint64_t D[6];
        st.block_bits(0, D[0], D[1]);
        st.block_bits(1, D[2], D[3]);
        st.block_bits(2, D[4], D[5]);
        auto draw = [&](int n) -> uint64_t {
            uint64_t r = 0;
#pragma unroll
            for (int q = 0; q < 6; ++q)
                if (q == n) r = D[q];
            if (n >= 6) {
                uint64_t x0, x1;
                st.block_bits((uint32_t)n >> 1, x0, x1);
                r = (n & 1) ? x1 : x0;
            }
            return r;
        };
        const int32_t nl = p.n1 + p.n2;
        const int32_t st2 = p.n2 > 0 ? p.start2 : b1;  // group 2 once a split exists
        const float l_smax = log2_pos(smax);
        const bool screen_b = screen && fabsf(l_smax) < 2.0f * LOG_RANGE;
        // per version: indices and slots (integer work only), then all the
        // versions' particle loads in flight together
        int32_t vi[V], vk[V], vsi[V], vsk[V], vnx[V];
        bool vfresh[V];
        // floor(U * n) for n = nl, nl + 1, ...: the exact products U 2^64 n
        // (128 bits) step by U 2^64 from one count to the next
        const uint64_t ai = D[0] & ~0xFFFull, ak = D[1] & ~0xFFFull;  // U * 2^64
        uint64_t ihi = __umul64hi(ai, (uint64_t)nl), ilo = ai * (uint64_t)nl;
        uint64_t khi = __umul64hi(ak, (uint64_t)nl), klo = ak * (uint64_t)nl;
#pragma unroll
        for (int v = 0; v < V; ++v) {
            const int32_t n = nl + v;
            if (v > 0) {
                ilo += ai;
                ihi += ilo < ai;
                klo += ak;
                khi += klo < ak;
            }
            int32_t i = -1, k = -2, nx = 2;
            if (valid) {
                // the FP64 product's rounding can only matter within half an
                // ulp of the next integer (floor_u52_times)
                i = ilo >= 0xFFFFFE0000000000ull ? floor_u52_times(D[0] >> 12, n) : (int32_t)ihi;
                k = klo >= 0xFFFFFE0000000000ull ? floor_u52_times(D[1] >> 12, n) : (int32_t)khi;
                int guard = 0;
                while (i == k && guard++ < (1 << 20)) k = floor_u52_times(draw(nx++) >> 12, n);
            }
            vi[v] = i;
            vk[v] = k;
            vnx[v] = nx;
            // a particle split off in this batch (index >= nl) is not written yet
            vfresh[v] = valid && (i >= nl || k >= nl);
            vsi[v] = i < p.n1 ? p.start1 + i : st2 + (i - p.n1);
            vsk[v] = k < p.n1 ? p.start1 + k : st2 + (k - p.n1);
        }
        PV va[V], vb[V];
#pragma unroll
        for (int v = 0; v < V; ++v) {
            if (valid && !vfresh[v]) {
                va[v] = P.wv[vsi[v]];
                vb[v] = P.wv[vsk[v]];
            } else {
                va[v] = PV{1.0, 0.0, 0.0, 0.0};
                vb[v] = va[v];
            }
        }
        // the scattering terms that depend on the draws alone, for the usual
        // draw positions (no redraw of k): they overlap the loads here instead
        // of lengthening the collision's dependent chain
        double sphi0, cphi0;
        sincos_2pi_u52(d.trig, D[3] >> 12, sphi0, cphi0);
        const double ct0 = fma(2.0, u52_to_double(D[4] >> 12), -1.0);
        const double sth0 = sqrt(1.0 - ct0 * ct0);
        // g^2, weights, screened and exact sigma g w per version
        bool vhas[V], vexact[V], veqw[V];
        double vg2[V], vsgw[V];
        float vls[V];
        double g0 = 0.0;
#pragma unroll
        for (int v = 0; v < V; ++v) {
            const PV& a = va[v];
            const PV& b = vb[v];
            const double gx = a.vx - b.vx, gy = a.vy - b.vy, gz = a.vz - b.vz;
            const double g2 = (gx * gx + gy * gy) + gz * gz;
            const double wm = dmax_pos(a.w, b.w);
            double sgw = -1.0;
            bool has = false, exact = false, have_g = false;
            double g = 0.0;
            float ls = 0.0f;
            if (valid && !vfresh[v]) {
                if ((uint64_t)__double_as_longlong(g2) > G2_TINY_BITS) {
                    has = true;
                } else {
                    g = sqrt(g2);
                    have_g = true;
                    has = g > EPS;
                }
                if (has) {
                    const float lw = log2_pos(wm), lg = log2_pos(g2);
                    ls = lC + lw + ex * lg;
                    exact = !screen_b || fabsf(lw) >= LOG_RANGE || fabsf(lg) >= LOG_RANGE ||
                            ls > l_smax - SCREEN_MARGIN;
                    if (exact) {
                        if (!have_g) g = sqrt(g2);
                        sgw = I.vhs_factor * pow(g, vexp) * g * wm;
                    }
                }
            }
            if (v == 0) g0 = sqrt(g2);
            veqw[v] = fabs(a.w - b.w) < dw_tol;  // an accepted collision without a split
            vg2[v] = g2;
            vsgw[v] = sgw;
            vhas[v] = has;
            vexact[v] = exact;
            vls[v] = ls;
        }
        // resolution in candidate order, one segment per version
        int s = 0, start = 0, end = -1;
        long long mrun = __double_as_longlong(smax);
        unsigned accm = 0u, splm = 0u;
        int myv = 0;
        bool myacc = false;
        int32_t ci = -1, ck = -1;  // this lane's particles once it is an accepted candidate
        while (end < 0) {
            int32_t i = 0, k = 0, nx = 2;
            bool fresh = false, has = false, exact = false, eqw = false;
            double g2 = 0.0, wm = 0.0, sgw = -1.0;
            float ls = 0.0f;
#pragma unroll
            for (int v = 0; v < V; ++v)
                if (v == s) {
                    i = vi[v];
                    k = vk[v];
                    nx = vnx[v];
                    fresh = vfresh[v];
                    has = vhas[v];
                    exact = vexact[v];
                    eqw = veqw[v];
                    g2 = vg2[v];
                    wm = dmax_pos(va[v].w, vb[v].w);
                    sgw = vsgw[v];
                    ls = vls[v];
                }
            const bool live = valid && gl >= start;
            // particles changed by accepted candidates of earlier segments
            bool conf = live && fresh;
            for (unsigned q = accm; q; q &= q - 1) {
                const int a = __ffs(q) - 1;
                const int32_t ta = grp.shfl(ci, a), tb = grp.shfl(ck, a);
                conf |= live && (i == ta || i == tb || k == ta || k == tb);
            }
            // running (sigma g w)_max (collision_ntc.jl:229) through this lane:
            // only exact values can raise it (screened ones lie below the
            // batch's starting maximum), so the scan visits those lanes only
            const long long key_me = max_key(sgw, live && has && exact);
            long long mk = mrun;
            for (unsigned q = grp.ballot(key_me >= 0); q; q &= q - 1) {
                const int e = __ffs(q) - 1;
                const long long ke = grp.shfl(key_me, e);
                if (gl >= e) mk = max(mk, ke);
            }
            const double m = __longlong_as_double(mk);
            // rand() < sigma_g_w / (sigma g w)_max (collision_ntc.jl:231)
            bool acc = false;
            if (live && has && !fresh) {
                const uint64_t um = draw(nx) >> 12;
                if (exact) {
                    acc = u52_to_double(um) < sgw / m;
                } else {
                    const float lm = log2_pos(m);
                    const float dl = ls - lm - log2_u52(um);
                    if (dl > SCREEN_MARGIN && fabsf(lm) < 2.0f * LOG_RANGE) {
                        acc = true;
                    } else if (dl >= -SCREEN_MARGIN || fabsf(lm) >= 2.0f * LOG_RANGE) {
                        const double g = sqrt(g2);
                        const double se = I.vhs_factor * pow(g, vexp) * g * wm;
                        acc = u52_to_double(um) < se / m;
                    }
                }
            }
            const bool spl = acc && !eqw;
            // particles changed by earlier accepted candidates of this segment
            const unsigned am = grp.ballot(acc);
            for (unsigned q = am; q; q &= q - 1) {
                const int a = __ffs(q) - 1;
                const int32_t ta = grp.shfl(i, a), tb = grp.shfl(k, a);
                if (gl > a) conf |= live && (i == ta || i == tb || k == ta || k == tb);
            }
            const unsigned cm = grp.ballot(conf), sm = grp.ballot(spl);
            const int fc = cm ? __ffs(cm) - 1 : G;
            const int fs = sm ? __ffs(sm) - 1 : G;
            const bool stop = fc <= fs;
            const int last = stop ? min(fc, nvalid) - 1 : fs;  // last lane of this segment
            if (last >= start) {
                const unsigned rng = (last - start + 1 >= 32 ? 0xFFFFFFFFu : ((1u << (last - start + 1)) - 1u)) << start;
                if (gl >= start && gl <= last) {
                    myv = s;
                    myacc = acc;
                    if (acc) {
                        ci = i;
                        ck = k;
                    }
                }
                accm |= am & rng;
                if (!stop) splm |= 1u << fs;
                mrun = grp.shfl(mk, last);
            }
            if (stop) {
                end = max(last + 1, start);
            } else {
                ++s;
                start = fs + 1;
                if (s == V || start >= nvalid) end = start;
            }
        }
        // the batch's accepted candidates collide, on disjoint particles
        const bool myspl = (splm >> gl) & 1u;
        if (myacc) {
            int32_t si = 0, sk = 0, nx = 2;
            double g2 = 0.0;
            PV a = va[0], b = vb[0];
#pragma unroll
            for (int v = 0; v < V; ++v)
                if (v == myv) {
                    si = vsi[v];
                    sk = vsk[v];
                    nx = vnx[v];
                    g2 = vg2[v];
                    a = va[v];
                    b = vb[v];
                }
            double wi = a.w, wk = b.w;  // weights after a split
            const double g = myv == 0 ? g0 : sqrt(g2);
            // compute_com! (collision_utils.jl:374-376)
            const double cx = I.mu1 * a.vx + I.mu2 * b.vx;
            const double cy = I.mu1 * a.vy + I.mu2 * b.vy;
            const double cz = I.mu1 * a.vz + I.mu2 * b.vz;
            if (myspl) {
                // split the heavier particle; the new particle keeps the
                // pre-collision velocity and position (collision_ntc.jl:235-267)
                const bool heavy_i = a.w > b.w;
                const int32_t src = heavy_i ? si : sk;
                const PV& h = heavy_i ? a : b;
                const double wl = heavy_i ? b.w : a.w;
                const int32_t ns_ = b1 + R.nsp1 + __popc(splm & ((1u << gl) - 1u));
                P.wv[ns_] = PV{h.w - wl, h.vx, h.vy, h.vz};
                cell[ns_] = c;
                key[ns_] = src;  // the position is copied after the loop
                if (heavy_i)
                    wi = wl;
                else
                    wk = wl;
            }
            // scatter_vhs! (collision_scattering.jl:17-29): phi = 2 pi rand(),
            // cos(theta) = 2 rand() - 1
            double sphi = sphi0, cphi = cphi0, ct = ct0, sth = sth0;
            if (nx != 2) {
                sincos_2pi_u52(d.trig, draw(nx + 1) >> 12, sphi, cphi);
                ct = fma(2.0, u52_to_double(draw(nx + 2) >> 12), -1.0);
                sth = sqrt(1.0 - ct * ct);
            }
            const double nxv = g * (sth * cphi), nyv = g * (sth * sphi), nzv = g * ct;
            P.wv[si] = PV{wi, cx + I.mu2 * nxv, cy + I.mu2 * nyv, cz + I.mu2 * nzv};
            P.wv[sk] = PV{wk, cx - I.mu1 * nxv, cy - I.mu1 * nyv, cz - I.mu1 * nzv};
        }
        const int nspl = __popc(splm);
        R.perf += __popc(accm);
        R.eqw += __popc(accm & ~splm);
        if (nspl) {
            if (p.n2 == 0) p.start2 = b1;
            p.n2 += nspl;
            R.nsp1 += nspl;
        }
        smax = __longlong_as_double(mrun);
        grp.sync();
        j0 += end;
    }
    // positions of the split-off particles: their parents', taken now.  A
    // parent split off earlier in this call has no position yet; its key
    // leads on to its own parent, and the first parent outside this call's
    // splits holds the position of the whole line.
    for (int32_t q = gl; q < R.nsp1; q += G) {
        int32_t src = key[b1 + q];
        for (int32_t h = 0; src >= b1 && src < b1 + R.nsp1 && h < R.nsp1; ++h) src = key[src];
        P.pos[b1 + q] = P.pos[src];
    }
    grp.sync();
    for (int32_t q = gl; q < R.nsp1; q += G) key[b1 + q] = c;
    grp.sync();
    R.smax = smax;
    return R;
}

// ------------------------------------------------------------------ props
struct CellMoments {
    double n, ux, uy, uz, T;
};

// Two-pass n, u, T of one (cell, species) list, one warp
// (compute_props!, physical_props.jl:104-154; sorted variant :317-354).
__device__ __forceinline__ CellMoments props_cell(const Cols& P, const Indexer& p, int32_t nl, double mass)
{
    const int lane = threadIdx.x & 31;
    double n = 0.0, sx = 0.0, sy = 0.0, sz = 0.0;
    for (int j = lane; j < nl; j += 32) {
        const PV r = P.wv[map_slot(p, j)];
        n += r.w;
        sx += r.vx * r.w;
        sy += r.vy * r.w;
        sz += r.vz * r.w;
    }
    n = warp_sum(n);
    sx = warp_sum(sx);
    sy = warp_sum(sy);
    sz = warp_sum(sz);
    CellMoments r;
    r.n = n;
    r.ux = r.uy = r.uz = r.T = 0.0;
    if (n > 0.0) {
        r.ux = sx / n;
        r.uy = sy / n;
        r.uz = sz / n;
        double E = 0.0;
        for (int j = lane; j < nl; j += 32) {
            const PV u = P.wv[map_slot(p, j)];
            const double dx = u.vx - r.ux, dy = u.vy - r.uy, dz = u.vz - r.uz;
            E = fma(u.w, (dx * dx + dy * dy) + dz * dz, E);
        }
        E = warp_sum(E);
        E *= 0.5 * mass / (n * K_B);
        r.T = (2.0 / 3.0) * E;
    }
    return r;
}

// Sums of four quantities over the warp in 6 additions instead of 20: the
// halves exchange two quantities, then quarters one, then a butterfly.
// Returns, in lanes 8q .. 8q+7, the warp total of a_q.
__device__ __forceinline__ double warp_sum4(double a0, double a1, double a2, double a3)
{
    const int lane = threadIdx.x & 31;
    const bool h16 = lane & 16, h8 = lane & 8;
    const double b0 = (h16 ? a2 : a0) + __shfl_xor_sync(0xFFFFFFFFu, h16 ? a0 : a2, 16);
    const double b1 = (h16 ? a3 : a1) + __shfl_xor_sync(0xFFFFFFFFu, h16 ? a1 : a3, 16);
    double c = (h8 ? b1 : b0) + __shfl_xor_sync(0xFFFFFFFFu, h8 ? b0 : b1, 8);
    c += __shfl_xor_sync(0xFFFFFFFFu, c, 4);
    c += __shfl_xor_sync(0xFFFFFFFFu, c, 2);
    c += __shfl_xor_sync(0xFFFFFFFFu, c, 1);
    return c;
}

// n, u, T of the group-1 lists of cells c0 .. c0 + nq - 1 (nq <= 32) of one
// species, one warp (compute_props_sorted!, physical_props.jl:317-354, and
// compute_props! for lists without group 2).  The same two passes as
// props_cell for every cell; the divisions and the final scaling run once for
// all nq cells, lane q finishing cell c0 + q, which returns its moments.
// props_cells_finish takes the first-pass sums of cell c0 + q in lane q (from
// props_pass1_into_lane, or from the sort's gather, which accumulates them in
// the same order) and runs the second pass.
__device__ __forceinline__ void props_pass1_into_lane(double n, double sx, double sy, double sz, int q, double& mn,
                                                      double& msx, double& msy, double& msz)
{
    const int lane = threadIdx.x & 31;
    const double t = warp_sum4(n, sx, sy, sz);
    const double tn = __shfl_sync(0xFFFFFFFFu, t, 0), tx = __shfl_sync(0xFFFFFFFFu, t, 8);
    const double ty = __shfl_sync(0xFFFFFFFFu, t, 16), tz = __shfl_sync(0xFFFFFFFFu, t, 24);
    if (lane == q) {
        mn = tn;
        msx = tx;
        msy = ty;
        msz = tz;
    }
}

__device__ __forceinline__ CellMoments props_cells_finish(const Cols& P, const Indexer* ind, int c0, int nq,
                                                          double mass, double mn, double msx, double msy, double msz,
                                                          unsigned skip = 0u)
{
    const int lane = threadIdx.x & 31;
    CellMoments r;
    r.n = mn;
    r.ux = r.uy = r.uz = r.T = 0.0;
    if (lane < nq && mn > 0.0) {
        r.ux = msx / mn;
        r.uy = msy / mn;
        r.uz = msz / mn;
    }
    double mE = 0.0;
    for (int q = 0; q < nq; ++q) {
        if ((skip >> q) & 1u) continue;
        const Indexer p = ind[c0 + q];
        const double ux = __shfl_sync(0xFFFFFFFFu, r.ux, q), uy = __shfl_sync(0xFFFFFFFFu, r.uy, q);
        const double uz = __shfl_sync(0xFFFFFFFFu, r.uz, q);
        double E = 0.0;
        // unrolled so that several records' loads are in flight (the sums
        // keep their order)
#pragma unroll 4
        for (int j = lane; j < p.n1; j += 32) {
            const PV u = P.wv[p.start1 + j];
            const double dx = u.vx - ux, dy = u.vy - uy, dz = u.vz - uz;
            E = fma(u.w, (dx * dx + dy * dy) + dz * dz, E);
        }
        E = warp_sum(E);
        if (lane == q) mE = E;
    }
    if (lane < nq && mn > 0.0) r.T = (2.0 / 3.0) * (mE * (0.5 * mass / (mn * K_B)));
    return r;
}

// cells with bit q of `skip` set are left out (their props come from a
// block-per-cell pass)
__device__ __forceinline__ CellMoments props_cells(const Cols& P, const Indexer* ind, int c0, int nq, double mass,
                                                   unsigned skip = 0u)
{
    const int lane = threadIdx.x & 31;
    double mn = 0.0, msx = 0.0, msy = 0.0, msz = 0.0;
    for (int q = 0; q < nq; ++q) {
        if ((skip >> q) & 1u) continue;
        const Indexer p = ind[c0 + q];
        double n = 0.0, sx = 0.0, sy = 0.0, sz = 0.0;
        for (int j = lane; j < p.n1; j += 32) {
            const PV r = P.wv[p.start1 + j];
            n += r.w;
            sx += r.vx * r.w;
            sy += r.vy * r.w;
            sz += r.vz * r.w;
        }
        props_pass1_into_lane(n, sx, sy, sz, q, mn, msx, msy, msz);
    }
    return props_cells_finish(P, ind, c0, nq, mass, mn, msx, msy, msz, skip);
}

// n, u, T of one large cell's group-1 list by a whole block (two passes as
// props_cell; the sums are combined per warp, then by thread 0 over the
// warps).  `red` is shared memory of 4 doubles per warp.  Valid in every
// thread.
__device__ __forceinline__ CellMoments props_cell_block(const Cols& P, const Indexer& p, double mass, double* red)
{
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
    const int nt = blockDim.x;
    double n = 0.0, sx = 0.0, sy = 0.0, sz = 0.0;
    // four records in flight per thread: a long list is latency-bound
    int j = tid;
    for (; j + 3 * nt < p.n1; j += 4 * nt) {
        PV r[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) r[u] = P.wv[p.start1 + j + u * nt];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            n += r[u].w;
            sx += r[u].vx * r[u].w;
            sy += r[u].vy * r[u].w;
            sz += r[u].vz * r[u].w;
        }
    }
    for (; j < p.n1; j += nt) {
        const PV r = P.wv[p.start1 + j];
        n += r.w;
        sx += r.vx * r.w;
        sy += r.vy * r.w;
        sz += r.vz * r.w;
    }
    const double t = warp_sum4(n, sx, sy, sz);
    if ((lane & 7) == 0) red[4 * wid + (lane >> 3)] = t;
    __syncthreads();
    double tn = 0.0, tx = 0.0, ty = 0.0, tz = 0.0;
    for (int w = 0; w < nw; ++w) {
        tn += red[4 * w];
        tx += red[4 * w + 1];
        ty += red[4 * w + 2];
        tz += red[4 * w + 3];
    }
    __syncthreads();
    CellMoments r;
    r.n = tn;
    r.ux = r.uy = r.uz = r.T = 0.0;
    if (tn > 0.0) {
        r.ux = tx / tn;
        r.uy = ty / tn;
        r.uz = tz / tn;
    }
    double E = 0.0;
    j = tid;
    for (; j + 3 * nt < p.n1; j += 4 * nt) {
        PV q[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) q[u] = P.wv[p.start1 + j + u * nt];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const double dx = q[u].vx - r.ux, dy = q[u].vy - r.uy, dz = q[u].vz - r.uz;
            E = fma(q[u].w, (dx * dx + dy * dy) + dz * dz, E);
        }
    }
    for (; j < p.n1; j += nt) {
        const PV u = P.wv[p.start1 + j];
        const double dx = u.vx - r.ux, dy = u.vy - r.uy, dz = u.vz - r.uz;
        E = fma(u.w, (dx * dx + dy * dy) + dz * dz, E);
    }
    E = warp_sum(E);
    if (lane == 0) red[wid] = E;
    __syncthreads();
    double tE = 0.0;
    for (int w = 0; w < nw; ++w) tE += red[w];
    __syncthreads();
    if (tn > 0.0) r.T = (2.0 / 3.0) * (tE * (0.5 * mass / (tn * K_B)));
    return r;
}

// ------------------------------------------------------------------ convection
struct WallView {
    const double2* trig;  // sector table of sincos_2pi_u52
    double L, min_x, max_x, inv_dx;
    long long bits_L, bits_min, bits_max;  // bit patterns of L, min_x, max_x (positive doubles order like integers)
    double vsq[2][MZ_MAX_SPECIES];
    double wv[2][3];
    double acc[2];
};

__device__ __forceinline__ void diffuse_reflect(Stream& st, const double2* trig, double& vx, double& vy, double& vz,
                                                double vsq, double normal, const double* wv)
{   // diffuse_reflection_x! (boundary_conditions.jl:79-93); the angle 2 pi rand()
    // through the scattering's table-driven sine and cosine
    double R = fmax(1e-50, st.uniform());
    const double vn = normal * sqrt(-vsq * log(R));
    R = fmax(1e-50, st.uniform());
    const double vt = sqrt(-vsq * log(R));
    double sR, cR;
    sincos_2pi_u52(trig, st.u52(), sR, cR);
    vx = vn + wv[0];
    vy = sR * vt + wv[1];
    vz = cR * vt + wv[2];
}

// Surface sampling of the two walls of a 1-D grid (SurfProps,
// surface_props.jl:22-67): element 0 = left wall (normal +x), 1 = right wall
// (normal -x); per element 11 sums: np, flux_incident, flux_reflected,
// force xyz, normal_pressure, shear_pressure xyz, kinetic_energy_flux.
// A thread keeps its sums in registers (constant indices) and a block flushes
// them with one atomic addition per quantity.
constexpr int SURF_Q = 11;

struct SurfAcc {
    double q[2][SURF_Q];
};

// update_surface_incident! (surface_props.jl:78-101, sign +1) and
// update_surface_reflected! (:113-134, sign -1) of element e
__device__ __forceinline__ void surf_update(SurfAcc& a, int e, double w, double vx, double vy, double vz,
                                            bool reflected)
{
    const double nx = e == 0 ? 1.0 : -1.0;
    const double px = w * vx, py = w * vy, pz = w * vz;
    const double pn = px * nx;
    const double sg = reflected ? -1.0 : 1.0;
    double u[SURF_Q];
    u[0] = reflected ? 0.0 : 1.0;
    u[1] = reflected ? 0.0 : w;
    u[2] = reflected ? -w : 0.0;
    u[3] = sg * px;
    u[4] = sg * py;
    u[5] = sg * pz;
    u[6] = -sg * pn;
    u[7] = sg * (px - pn * nx);
    u[8] = sg * py;
    u[9] = sg * pz;
    u[10] = sg * (0.5 * (px * vx + py * vy + pz * vz));
#pragma unroll
    for (int k = 0; k < SURF_Q; ++k) {
        a.q[0][k] += e == 0 ? u[k] : 0.0;
        a.q[1][k] += e == 1 ? u[k] : 0.0;
    }
}

// block sum of every thread's SurfAcc into dst[2][SURF_Q] (one atomic per
// quantity per block); all threads of the block call it
__device__ __forceinline__ void surf_flush(const SurfAcc& a, double* dst, bool any)
{
    __shared__ double part[2 * SURF_Q];
    __shared__ int active;
    if (threadIdx.x == 0) active = 0;
    if (threadIdx.x < 2 * SURF_Q) part[threadIdx.x] = 0.0;
    __syncthreads();
    if (__any_sync(0xFFFFFFFFu, any) && (threadIdx.x & 31) == 0) atomicOr(&active, 1);
    __syncthreads();
    if (active) {
#pragma unroll
        for (int e = 0; e < 2; ++e)
#pragma unroll
            for (int k = 0; k < SURF_Q; ++k) {
                const double v = warp_sum(a.q[e][k]);
                if ((threadIdx.x & 31) == 0 && v != 0.0) atomicAdd(&part[e * SURF_Q + k], v);
            }
        __syncthreads();
        if (threadIdx.x < 2 * SURF_Q && part[threadIdx.x] != 0.0) atomicAdd(&dst[threadIdx.x], part[threadIdx.x]);
    }
}

// wall-hit loop of convect_single_particle! (convection_1D.jl:22-42); returns hits
__device__ __forceinline__ int convect_walls(Stream& st, const WallView& W, int s, double& x, double& vx, double& vy,
                                             double& vz, double dt, bool& cap, SurfAcc* surf = nullptr, double w = 0.0)
{
    double t_rest = dt;
    double x_old = x;
    double x_new = fma(vx, dt, x);
    int hits = 0;
    while ((x_new >= W.L) || (x_new <= 0.0)) {
        if (hits >= 1000) {
            cap = true;
            break;
        }
        ++hits;
        int bc;
        double normal;
        if (x_new >= W.L) {
            t_rest -= fabs((W.L - x_old) / vx);
            bc = 1;
            normal = -1.0;
            x_old = W.L;
        } else {
            t_rest -= fabs(x_old / vx);
            bc = 0;
            normal = 1.0;
            x_old = 0.0;
        }
        if (surf) surf_update(*surf, bc, w, vx, vy, vz, false);
        // reflect_particle_x! (boundary_conditions.jl:108-121)
        const double acc = W.acc[bc];
        if (acc == 0.0) {
            vx = -vx;
        } else if (acc == 1.0) {
            diffuse_reflect(st, W.trig, vx, vy, vz, W.vsq[bc][s], normal, W.wv[bc]);
        } else {
            if (st.uniform() < acc)
                diffuse_reflect(st, W.trig, vx, vy, vz, W.vsq[bc][s], normal, W.wv[bc]);
            else
                vx = -vx;
        }
        if (surf) surf_update(*surf, bc, w, vx, vy, vz, true);
        x_new = fma(vx, t_rest, x_old);
    }
    x = fmin(fmax(x_new, W.min_x), W.max_x);
    return hits;
}

// get_cell (grid_uniform1D.jl:97-99), 0-based, clamped with a status flag
__device__ __forceinline__ int32_t cell_of(const DomainView& d, double x, double inv_dx)
{
    int32_t k = __double2int_rd(x * inv_dx);
    if (k < 0 || k >= d.n_cells) {
        set_status(d, ST_OUTSIDE_GRID);
        k = k < 0 ? 0 : d.n_cells - 1;
    }
    return k;
}

// x + vx*dt for a particle that stays inside (0, L): the clamp of
// convect_single_particle! (convection_1D.jl:44-46).  Returns false when the
// new position hits a wall: x_new >= L or x_new <= 0 (the comparisons are made
// on the bit patterns, where doubles of one sign order like integers).
__device__ __forceinline__ bool move_free(const WallView& W, double xn, double& x)
{
    const long long b = __double_as_longlong(xn);
    if (b <= 0 || b >= W.bits_L) return false;
    x = b < W.bits_min ? W.min_x : (b > W.bits_max ? W.max_x : xn);
    return true;
}

__host__ inline void wall_bits(WallView& W)
{
    memcpy(&W.bits_L, &W.L, 8);
    memcpy(&W.bits_min, &W.min_x, 8);
    memcpy(&W.bits_max, &W.max_x, 8);
}

}  // namespace mz
