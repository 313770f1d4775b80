// SWPM collisions of variable-weight particles of one species: swpm!
// (collision_swpm.jl:201-288) with compute_n_coll_single_species (:170-173),
// VHS cross-sections and scatter_vhs! (collision_scattering.jl:17-29).
//
// A collision of particles i, k with weights w_i, w_k takes
// dw = min(w_i, w_k) / (1 + G) from both and appends two particles of weight
// dw: copies of i and k (positions and velocities) that then scatter.  The
// candidate count uses (sigma g)_max * w_max * (G + 1), and a candidate is
// accepted with probability sigma g max(w_i, w_k) / (w_max (sigma g)_max).
//
// One group of G lanes owns one cell and keeps the reference's sequential
// candidate loop exactly, like the NTC kernels (ntc.cu):
//   * candidate j draws from its own stream (i, k, retries of k, acceptance,
//     scattering angles -- the reference's order; the NTC streams);
//   * a batch ends before the first candidate that shares a particle with an
//     earlier candidate of the batch, and right after the first accepted
//     candidate: its two new particles change the cell's count, which later
//     index draws multiply by, and their weights change later tests;
//   * an inclusive max-scan of sigma*g over the batch gives every candidate
//     the running (sigma g)_max it is tested against.
// New particles go to the cell's group 2 inside a region of 2 n_coll slots
// reserved per cell (an exclusive scan of the reservations).
#include "cell_ops.cuh"
#include "mz_host.h"

#include <algorithm>

using namespace mz;

namespace {

// compute_n_coll_single_species for SWPM (collision_swpm.jl:170-173); resets
// the per-call counters like swpm! (:225-230)
__device__ __forceinline__ int32_t swpm_ncoll(const DomainView& d, CollisionFactors& cf, int64_t n, double w_max,
                                              double G, double dt, double V, uint64_t seed, uint32_t pc, uint32_t stp,
                                              uint32_t rid)
{
    Stream st;
    st.init(seed, TAG_NCOLL, pc, stp, rid, 0);
    const double U = st.uniform();
    const double f = 0.5 * dt * (double)n * (double)(n - 1) * cf.smax * w_max * (G + 1.0) / V + U;
    double fl = floor(f);
    if (!(fl < 1.0e8)) {
        set_status(d, ST_CAPACITY);
        fl = fl != fl ? 0.0 : 1.0e8;
    }
    const int32_t nci = (int32_t)fl;
    cf.n1 = (int32_t)n;
    cf.n2 = (int32_t)n;
    cf.n_coll = nci;
    cf.n_coll_performed = 0;
    cf.n_eq_w_coll_performed = 0;
    cf.n_split = 0;
    return nci;
}

// maximum weight of a cell's particles (swpm!, collision_swpm.jl:204-218), by
// the lanes of a group of width W; weights are >= 0, so bit patterns order them
template <int W>
__device__ __forceinline__ double cell_w_max(const Cols& P, const Indexer& p, int rank, unsigned mask)
{
    const int32_t nl = p.n1 + p.n2;
    long long m = 0;
    for (int32_t j = rank; j < nl; j += W) m = max(m, (long long)__double_as_longlong(P.wv[map_slot(p, j)].w));
#pragma unroll
    for (int o = W / 2; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(mask, m, o, W));
    return __longlong_as_double(m);
}

// The candidate loop of swpm! for one cell, by one group of G lanes (all
// lanes call it with identical arguments).  Returns the running maximum, the
// number of accepted collisions (perf) and of appended particles (nsp1).
template <int G>
__device__ __forceinline__ NtcResult swpm_cell(const DomainView& d, const Interaction& I, int c, int32_t ncoll,
                                               double smax, double inv_w_max, double wtf, const Cols& P, Indexer& p,
                                               int32_t* cellv, int32_t* key, int32_t b, uint64_t seed, uint32_t pc,
                                               uint32_t stp, uint32_t rid)
{
    const WarpGroup<G> grp;
    const int gl = grp.rank;
    const double vexp = fma(-2.0, I.vhs_o, 1.0);  // sigma_vhs exponent, collision_cross_sections.jl:179-181
    NtcResult R;
    R.perf = R.eqw = R.nsp1 = R.nsp2 = 0;
    for (int32_t j0 = 0; j0 < ncoll;) {
        const int32_t j = j0 + gl;
        const bool valid = j < ncoll;
        Stream st;
        st.init(seed, TAG_CAND, pc, stp, rid, (uint32_t)j);
        int32_t i = -1, k = -2;
        if (valid) {
            // i, k = floor(rand() * n_local), k redrawn while equal (collision_swpm.jl:236-241)
            const int32_t nl = p.n1 + p.n2;
            i = floor_u52_times(st.u52(), nl);
            k = floor_u52_times(st.u52(), nl);
            int guard = 0;
            while (i == k && guard++ < (1 << 20)) k = floor_u52_times(st.u52(), nl);
        }
        bool conflict = false;
#pragma unroll
        for (int src = 0; src < G - 1; ++src) {
            const int32_t ii = grp.shfl(i, src);
            const int32_t kk = grp.shfl(k, src);
            if (src < gl) conflict |= (ii == i) | (ii == k) | (kk == i) | (kk == k);
        }
        const unsigned cm = grp.ballot(valid && conflict);
        const int nvalid = min(G, ncoll - j0);
        int B = cm ? min(nvalid, __ffs(cm) - 1) : nvalid;
        const bool act = gl < B;

        int32_t si = 0, sk = 0;
        PV a, bb;
        a.w = bb.w = 0.0;
        double g = 0.0, sg = -1.0;
        bool has = false;
        if (act) {
            si = map_slot(p, i);
            sk = map_slot(p, k);
            a = P.wv[si];
            bb = P.wv[sk];
            // compute_g! (collision_utils.jl:388-391) and g > eps() (collision_swpm.jl:253)
            const double gx = a.vx - bb.vx, gy = a.vy - bb.vy, gz = a.vz - bb.vz;
            g = sqrt((gx * gx + gy * gy) + gz * gz);
            has = g > EPS;
            if (has) sg = I.vhs_factor * pow(g, vexp) * g;  // sigma_vhs(g) * g
        }
        // running (sigma g)_max (collision_swpm.jl:259) as an inclusive max-scan
        long long mk = max_key(sg, act && has);
#pragma unroll
        for (int o = 1; o < G; o <<= 1) {
            const long long t = grp.up(mk, o);
            if (gl >= o) mk = max(mk, t);
        }
        mk = max(mk, __double_as_longlong(smax));
        const double m = __longlong_as_double(mk);
        bool acc = false;
        if (act && has) {
            // rand() < sigma g max(w_i, w_k) / w_max / (sigma g)_max (collision_swpm.jl:261)
            const double wm = dmax_pos(a.w, bb.w);
            acc = u52_to_double(st.u52()) < sg * wm * inv_w_max / m;
        }
        const unsigned am = grp.ballot(acc);
        if (am) B = min(B, __ffs(am));  // the batch ends after the first accepted candidate
        if (am && gl == B - 1) {
            // compute_com! (collision_utils.jl:374-376)
            const double cx = I.mu1 * a.vx + I.mu2 * bb.vx;
            const double cy = I.mu1 * a.vy + I.mu2 * bb.vy;
            const double cz = I.mu1 * a.vz + I.mu2 * bb.vz;
            // weight transfer and the two new particles (collision_swpm.jl:268-281)
            const double dw = fmin(a.w, bb.w) * wtf;
            P.wv[si].w = a.w - dw;
            P.wv[sk].w = bb.w - dw;
            const int32_t n0 = b + R.nsp1, n1 = n0 + 1;
            P.pos[n0] = P.pos[si];
            P.pos[n1] = P.pos[sk];
            // scatter_vhs! of the new pair (collision_swpm.jl:282-283)
            double sphi, cphi;
            sincos_2pi_u52(d.trig, st.u52(), sphi, cphi);
            const double ct = fma(2.0, st.uniform(), -1.0);
            const double sth = sqrt(1.0 - ct * ct);
            const double nx = g * (sth * cphi), ny = g * (sth * sphi), nz = g * ct;
            P.wv[n0] = PV{dw, cx + I.mu2 * nx, cy + I.mu2 * ny, cz + I.mu2 * nz};
            P.wv[n1] = PV{dw, cx - I.mu1 * nx, cy - I.mu1 * ny, cz - I.mu1 * nz};
            cellv[n0] = c;
            cellv[n1] = c;
            key[n0] = c;
            key[n1] = c;
        }
        smax = __longlong_as_double(grp.shfl(mk, B - 1));
        if (am) {
            R.perf += 1;
            if (p.n2 == 0) p.start2 = b;
            p.n2 += 2;
            R.nsp1 += 2;
        }
        grp.sync();
        j0 += B;
    }
    R.smax = smax;
    return R;
}

// per cell: w_max, n_coll and a reservation of 2 n_coll slots (0 outside the
// range; every cell is written because the scan reads all), one warp per cell
__global__ void k_swpm_prepare(DomainView d, int s, uint32_t pc, int cfi, double G, double dt, int cb, int ce,
                               uint32_t step, int32_t* res)
{
    const SpeciesView& S = d.sp[s];
    const int lane = threadIdx.x & 31;
    const int nw = (int)((gridDim.x * blockDim.x) >> 5);
    for (int c = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); c < d.n_cells; c += nw) {
        int32_t r = 0;
        if (c >= cb && c < ce) {
            const Indexer p = S.ind[c];
            const double w_max = cell_w_max<32>(S.A, p, lane, 0xFFFFFFFFu);
            if (lane == 0) {
                CollisionFactors& cf = d.cf[(size_t)cfi * d.n_cells + c];
                r = 2 * swpm_ncoll(d, cf, p.n1 + p.n2, w_max, G, dt, d.cell_V[c], cell_seed(d, c), pc,
                                   cell_step(d, c, step), cell_rid(d, c));
            }
        }
        if (lane == 0) res[c] = r;
    }
}

template <int G>
__global__ void __launch_bounds__(256) k_swpm(DomainView d, int s, uint32_t pc, int cfi, int cb, int ce,
                                              uint32_t step, double wtf, const int32_t* base, const int32_t* res)
{
    const SpeciesView& S = d.sp[s];
    const Interaction I = d.inter[s + d.n_species * s];
    const WarpGroup<G> grp;
    const int ngroups = (gridDim.x * blockDim.x) / G;
    for (int c = cb + (int)((blockIdx.x * blockDim.x + threadIdx.x) / G); c < ce; c += ngroups) {
        CollisionFactors* cfp = &d.cf[(size_t)cfi * d.n_cells + c];
        const int32_t ncoll = cfp->n_coll;
        const int32_t b = base[c];
        int32_t used = 0;
        if (ncoll > 0) {
            Indexer p = S.ind[c];
            const double w_max = cell_w_max<G>(S.A, p, grp.rank, grp.mask);
            const NtcResult R = swpm_cell<G>(d, I, c, ncoll, cfp->smax, 1.0 / w_max, wtf, S.A, p, S.cell, S.key, b,
                                             cell_seed(d, c), pc, cell_step(d, c, step), cell_rid(d, c));
            used = R.nsp1;
            if (grp.rank == 0) {
                cfp->smax = R.smax;
                cfp->n_coll_performed = R.perf;
                cfp->n_split = R.nsp1;
                S.ind[c] = p;
                atomicAdd(&d.counters->candidates, (unsigned long long)ncoll);
                atomicAdd(&d.counters->accepted, (unsigned long long)R.perf);
                atomicAdd(&d.counters->splits, (unsigned long long)R.nsp1);
            }
        }
        // reserved slots not taken by new particles become dead
        const int32_t r = res[c];
        for (int32_t q = used + grp.rank; q < r; q += G) S.cell[b + q] = -1;
    }
}

}  // namespace

void launch_swpm(mz_domain* d, int s, double G, double dt, int64_t cb, int64_t ce, uint64_t step)
{
    mz_ctx* c = d->ctx;
    const uint32_t pc = (uint32_t)(s * d->ns + s);
    const int cfi = s + d->ns * s;
    launch_compact(d, s);
    SpeciesHost& A = d->sp[s];
    DomainView v = make_view(d);
    const int64_t nc = d->n_cells;
    const int pblocks = (int)std::max<int64_t>(1, std::min<int64_t>(div_up(nc * 32, 256), (int64_t)c->num_sms * 8));
    MZ_LAUNCH(c, "swpm_prepare", k_swpm_prepare, pblocks, 256, 0, v, s, pc, cfi, G, dt, (int)cb, (int)ce,
              (uint32_t)step, A.fill);
    launch_scan_cells(d, A.fill, A.ind, A.fill, d->d_scalar, false, A.work, A.hw);
    MZ_CK(cudaMemcpyAsync(d->h_scalar, d->d_scalar, sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
    MZ_CK(cudaStreamSynchronize(c->stream));
    const int64_t tot = d->h_scalar[0];
    if (A.hw + tot > A.capacity) reserve_species(d, s, A.hw + tot + 256);
    v = make_view(d);
    const int Gw = ntc_group_width(ce - cb);
    const int blocks =
        (int)std::max<int64_t>(1, std::min<int64_t>(div_up(std::max<int64_t>(1, ce - cb) * Gw, 256),
                                                    (int64_t)c->num_sms * 16));
    using KSwpm = void (*)(DomainView, int, uint32_t, int, int, int, uint32_t, double, const int32_t*, const int32_t*);
    const KSwpm kern = Gw == 8 ? k_swpm<8> : Gw == 16 ? k_swpm<16> : k_swpm<32>;
    MZ_LAUNCH(c, "swpm", kern, blocks, 256, 0, v, s, pc, cfi, (int)cb, (int)ce, (uint32_t)step, 1.0 / (1.0 + G),
              A.work, A.fill);
    A.hw += tot;
    A.compact = false;
    A.group2 = true;
    // the live total from the indexers
    std::vector<mz::Indexer> ind(d->n_cells);
    MZ_CK(cudaMemcpyAsync(ind.data(), A.ind, d->n_cells * sizeof(mz::Indexer), cudaMemcpyDeviceToHost, c->stream));
    MZ_CK(cudaStreamSynchronize(c->stream));
    int64_t n = 0;
    for (auto& p : ind) n += p.n1 + p.n2;
    A.n_total = n;
}

extern "C" int mz_swpm(mz_domain* d, int32_t s, double G, double dt, int64_t cb, int64_t ce, uint64_t step)
{
    API_TRY
    MZ_REQUIRE(d && s >= 0 && s < d->ns, "mz_swpm: bad species");
    MZ_REQUIRE(cb >= 0 && ce <= d->n_cells && cb <= ce, "mz_swpm: bad cell range");
    MZ_REQUIRE(G >= 0.0, "mz_swpm: G must be non-negative");
    MZ_CK(cudaSetDevice(d->ctx->device));
    if (cb == ce) return MZ_OK;
    launch_swpm(d, s, G, dt, cb, ce, step);
    check_status(d);
    API_CATCH(d->ctx)
}
