/*
 * ORACLE -- test infrastructure, NOT product code.
 *
 * A plain C++ restatement of Merzbild.jl's per-step DSMC hot path (reference
 * v0.7.10, Julia; the reference itself cannot run in this environment because
 * no Julia toolchain exists).  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline legs of bench.py may load this library, and only as the
 * result the device is compared against or as the timed CPU baseline.  The
 * product library never links or calls it.
 *
 * Every function follows one reference function (file:line in the reference
 * repository is given beside it).  Data layout mirrors the reference: AoS
 * Particle records, a ParticleVector with `index` indirection, `cell` array and
 * LIFO `buffer`, and a ParticleIndexerArray whose fields are 1-based exactly
 * like the reference (empty group: start = 0, end = -1).
 *
 * Deviations, all deliberate and shared with the device library:
 *   * RNG: counter-based Philox streams (philox_ref.h) instead of one
 *     sequential Julia stream; the draw ORDER inside each unit is kept.
 *   * @muladd contractions of scalar a*b+c in the reference become explicit
 *     std::fma here (SVector expressions are not fused by MuladdMacro's
 *     generic fallback and stay unfused here as well).  The file is compiled
 *     with -ffp-contract=off so no other contraction happens on any host.
 *   * convect_single_particle!: the wall-hit loop is capped at
 *     ORC_MAX_WALL_HITS iterations (the reference loops forever if a particle
 *     lands exactly on a wall with zero remaining time).
 *   * samplers use log(1 - U) instead of log(U) so that U == 0 cannot produce
 *     an infinite speed (same distribution).
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "philox_ref.h"

namespace {

const double k_B = 1.380649e-23;                 // constants.jl:4
const double twopi = 2.0 * 3.141592653589793;    // constants.jl:29
const double PI = 3.141592653589793;
const int64_t DELTA_PARTICLES = 256;             // Merzbild.jl:23
const int ORC_MAX_WALL_HITS = 1000;

struct Particle {                                // particles.jl:14-18
    double w;
    double v[3];
    double x[3];
};

struct ParticleIndexer {                         // particles.jl:56-66
    int64_t n_local, start1, end1, n_group1, start2, end2, n_group2;
};

struct ParticleVector {                          // particles.jl:194-200
    std::vector<Particle> particles;
    std::vector<int64_t> index;   // 1-based values
    std::vector<int64_t> cell;
    std::vector<int64_t> buffer;
    int64_t nbuffer = 0;

    Particle& at(int64_t i) { return particles[index[i - 1] - 1]; }  // getindex, particles.jl:225-227
    int64_t length() const { return (int64_t)particles.size(); }
};

struct Interaction {                             // collision_utils.jl:73-82
    double m_r, mu1, mu2, vhs_d, vhs_o, vhs_Tref, vhs_muref, vhs_factor;
};

struct CollisionFactors {                        // collision_ntc.jl:18-25
    int64_t n1 = 0, n2 = 0;
    double sigma_g_w_max = 0.0;
    int64_t n_coll = 0, n_coll_performed = 0, n_eq_w_coll_performed = 0;
};

struct Orc {
    int64_t n_cells;
    int32_t n_species;
    std::vector<ParticleVector> pv;
    std::vector<ParticleIndexer> indexer;        // [(cell-1) + n_cells * s]
    std::vector<int64_t> n_total;
    std::vector<uint8_t> contiguous;
    std::vector<double> mass;
    std::vector<Interaction> inter;              // [s1 + ns * s2]
    std::vector<CollisionFactors> cf;            // [s1 + ns * (s2 + ns * (cell-1))]
    // global id of cell 1 minus one: a slab of a larger grid keys the
    // collision, convection and merge streams of its cell c on c - 1 + cell_offset
    int64_t cell_offset = 0;

    ParticleIndexer& pi(int64_t cell, int s) { return indexer[(cell - 1) + n_cells * s]; }
    CollisionFactors& cfa(int s1, int s2, int64_t cell) {
        return cf[s1 + n_species * (s2 + n_species * (cell - 1))];
    }
};

ParticleIndexer empty_indexer() { return ParticleIndexer{0, 0, -1, 0, 0, -1, 0}; }  // particles.jl:84

// ---------------------------------------------------------------- particles.jl
void pv_init(ParticleVector& pv, int64_t np)     // ParticleVector(np), particles.jl:210-212
{
    pv.particles.assign(np, Particle{0.0, {0, 0, 0}, {0, 0, 0}});
    pv.index.resize(np);
    pv.cell.assign(np, 0);
    pv.buffer.resize(np);
    for (int64_t i = 0; i < np; ++i) {
        pv.index[i] = i + 1;
        pv.buffer[i] = np - i;
    }
    pv.nbuffer = np;
}

void pv_resize(ParticleVector& pv, int64_t n)    // Base.resize!, particles.jl:269-298
{
    int64_t old_len = pv.length();
    pv.particles.resize(n, Particle{0.0, {0, 0, 0}, {0, 0, 0}});
    pv.index.resize(n);
    pv.cell.resize(n, 0);
    std::vector<int64_t> old_buf(pv.buffer.begin(), pv.buffer.begin() + old_len);
    pv.buffer.resize(n);
    int64_t n_diff = n - old_len;
    for (int64_t i = old_len + 1; i <= n; ++i) {
        pv.particles[i - 1] = Particle{0.0, {0, 0, 0}, {0, 0, 0}};
        pv.index[i - 1] = i;
    }
    for (int64_t i = 0; i < old_len; ++i) pv.buffer[n_diff + i] = old_buf[i];
    for (int64_t i = 1; i <= n_diff; ++i) pv.buffer[i - 1] = n + 1 - i;
    pv.nbuffer += n_diff;
}

inline void update_particle_buffer_new_particle(ParticleVector& pv, int64_t position)  // particles.jl:311-315
{
    pv.index[position - 1] = pv.buffer[pv.nbuffer - 1];
    pv.nbuffer -= 1;
}

inline int64_t map_cont_index(const ParticleIndexer& p, int64_t i)  // particles.jl:364-366
{
    return i < p.n_group1 ? i + p.start1 : (i - p.n_group1) + p.start2;
}

inline void update_particle_indexer_new_particle(Orc& o, int64_t cell, int s)  // particles.jl:426-433
{
    o.n_total[s] += 1;
    ParticleIndexer& p = o.pi(cell, s);
    p.n_local += 1;
    p.n_group2 += 1;
    p.start2 = p.start2 > 0 ? p.start2 : o.n_total[s];
    p.end2 = o.n_total[s];
}

inline void update_buffer_index_new_particle(Orc& o, int64_t cell, int s)  // particles.jl:718-721
{
    update_particle_indexer_new_particle(o, cell, s);
    update_particle_buffer_new_particle(o.pv[s], o.n_total[s]);
}

void delete_particle_end_group1(Orc& o, int64_t cell, int s)  // particles.jl:501-525
{
    ParticleIndexer& p = o.pi(cell, s);
    ParticleVector& pv = o.pv[s];
    if (p.n_group1 == 0) return;
    int64_t index_of_deleted = p.end1;
    pv.at(index_of_deleted).w = 0.0;
    p.n_local -= 1;
    p.end1 -= 1;
    p.n_group1 -= 1;
    o.n_total[s] -= 1;
    if (p.end1 < p.start1) {
        p.start1 = 0;
        p.end1 = -1;
    }
    pv.nbuffer += 1;
    pv.buffer[pv.nbuffer - 1] = pv.index[index_of_deleted - 1];
}

void delete_particle_end_group2(Orc& o, int64_t cell, int s)  // particles.jl:542-566
{
    ParticleIndexer& p = o.pi(cell, s);
    ParticleVector& pv = o.pv[s];
    if (p.n_group2 == 0) return;
    int64_t index_of_deleted = p.end2;
    pv.at(index_of_deleted).w = 0.0;
    p.n_local -= 1;
    p.end2 -= 1;
    p.n_group2 -= 1;
    o.n_total[s] -= 1;
    if (p.end2 < p.start2) {
        p.start2 = 0;
        p.end2 = -1;
    }
    pv.nbuffer += 1;
    pv.buffer[pv.nbuffer - 1] = pv.index[index_of_deleted - 1];
}

void delete_particle_end(Orc& o, int64_t cell, int s)  // particles.jl:478-484
{
    if (o.pi(cell, s).n_group2 > 0)
        delete_particle_end_group2(o, cell, s);
    else
        delete_particle_end_group1(o, cell, s);
}

void squash_pia(Orc& o, int s)                   // particles.jl:622-682
{
    if (o.contiguous[s]) return;
    ParticleVector& pv = o.pv[s];
    int64_t n_cells = o.n_cells;
    auto move = [&](int64_t j, int64_t offset) {
        pv.index[j - 1] = pv.index[j + offset - 1];
        pv.cell[j - 1] = pv.cell[j + offset - 1];
    };
    if (n_cells == 1) {
        ParticleIndexer& p = o.pi(1, s);
        if (p.n_group2 > 0) {
            int64_t e1 = p.end1 > 0 ? p.end1 : 0;
            int64_t offset = p.start2 - (e1 + 1);
            if (offset > 0) {
                p.start2 -= offset;
                p.end2 -= offset;
                for (int64_t j = p.start2; j <= p.end2; ++j) move(j, offset);
            }
        }
    } else {
        int64_t last_end = o.pi(1, s).end1 > 0 ? o.pi(1, s).end1 : 0;
        for (int64_t i = 1; i <= n_cells - 1; ++i) {
            ParticleIndexer& p = o.pi(i + 1, s);
            int64_t offset = p.start1 - (last_end + 1);
            if (offset > 0) {
                p.start1 -= offset;
                p.end1 -= offset;
                for (int64_t j = p.start1; j <= p.end1; ++j) move(j, offset);
            }
            last_end = p.end1 > 0 ? p.end1 : last_end;
        }
        for (int64_t i = 1; i <= n_cells; ++i) {
            ParticleIndexer& p = o.pi(i, s);
            if (p.n_group2 > 0) {
                int64_t offset = p.start2 - (last_end + 1);
                if (offset > 0) {
                    p.start2 -= offset;
                    p.end2 -= offset;
                    for (int64_t j = p.start2; j <= p.end2; ++j) move(j, offset);
                }
                last_end = p.end2 > 0 ? p.end2 : last_end;
            }
        }
    }
    o.contiguous[s] = 1;
}

void restore_particle_ordering(ParticleVector& pv)  // particles.jl:1086-1137
{
    int64_t n_total = (int64_t)pv.index.size();
    int64_t n_used = n_total - pv.nbuffer;
    std::vector<int64_t> inv_map(n_total, 0);
    for (int64_t i = 1; i <= n_used; ++i) inv_map[pv.index[i - 1] - 1] = i;
    for (int64_t i = 1; i <= n_used; ++i) {
        int64_t cur = pv.index[i - 1];
        if (cur != i) {
            int64_t displaced = inv_map[i - 1];
            std::swap(pv.particles[i - 1], pv.particles[cur - 1]);
            pv.index[i - 1] = i;
            inv_map[i - 1] = i;
            if (displaced > 0) {
                pv.index[displaced - 1] = cur;
                inv_map[cur - 1] = displaced;
            } else {
                inv_map[cur - 1] = 0;
            }
        }
    }
    for (int64_t i = n_used + 1; i <= n_total; ++i) pv.index[i - 1] = i;
    for (int64_t i = 1; i <= pv.nbuffer; ++i) pv.buffer[i - 1] = n_total - i + 1;
}

// ---------------------------------------------------------- collision_utils.jl
double compute_vhs_factor(double Tref, double d, double o, double m_r)  // collision_utils.jl:98-101
{
    return PI * (d * d) * std::pow(2.0 * k_B * Tref / m_r, o - 0.5) / std::tgamma(2.5 - o);
}

double compute_mu_ref(double m_r, double o, double Tref, double d)  // collision_utils.jl:218-223
{
    double numerator = 30.0 * std::sqrt(m_r * k_B * Tref);
    double denominator = 4.0 * std::sqrt(PI) * (5.0 - 2.0 * o) * (7.0 - 2.0 * o) * d * d;
    return numerator / denominator;
}

inline double sigma_vhs(const Interaction& I, double g)  // collision_cross_sections.jl:179-181
{
    return I.vhs_factor * std::pow(g, std::fma(-2.0, I.vhs_o, 1.0));
}

double estimate_sigma_g_w_max(const Interaction& I, double m1, double m2, double T1, double T2, double Fnum,
                              double mult)    // collision_utils.jl:418-423
{
    double g1 = std::sqrt(2.0 * T1 * k_B / m1);
    double g2 = std::sqrt(2.0 * T2 * k_B / m2);
    double g = 0.5 * (g1 + g2);
    return mult * sigma_vhs(I, g) * g * Fnum;
}

struct CollisionData {                           // collision_utils.jl:22-31 (fields used on the path)
    double v_com[3];
    double g;
    double g_vec[3];
    double g_vec_new[3];
};

inline void compute_g(CollisionData& cd, const Particle& p1, const Particle& p2)  // collision_utils.jl:388-391
{
    for (int c = 0; c < 3; ++c) cd.g_vec[c] = p1.v[c] - p2.v[c];
    cd.g = std::sqrt((cd.g_vec[0] * cd.g_vec[0] + cd.g_vec[1] * cd.g_vec[1]) + cd.g_vec[2] * cd.g_vec[2]);
}

inline void compute_com(CollisionData& cd, const Interaction& I, const Particle& p1, const Particle& p2)
{   // collision_utils.jl:374-376 (SVector muladd: generic, unfused)
    for (int c = 0; c < 3; ++c) cd.v_com[c] = I.mu1 * p1.v[c] + I.mu2 * p2.v[c];
}

inline void scatter_vhs(orc_stream* rng, CollisionData& cd, const Interaction& I, Particle& p1, Particle& p2)
{   // collision_scattering.jl:17-29
    double phi = twopi * orc_stream_uniform(rng);
    double cphi = std::cos(phi);
    double sphi = std::sin(phi);
    double ctheta = std::fma(2.0, orc_stream_uniform(rng), -1.0);
    double stheta = std::sqrt(1.0 - ctheta * ctheta);
    cd.g_vec_new[0] = cd.g * (stheta * cphi);
    cd.g_vec_new[1] = cd.g * (stheta * sphi);
    cd.g_vec_new[2] = cd.g * ctheta;
    for (int c = 0; c < 3; ++c) {
        p1.v[c] = cd.v_com[c] + I.mu2 * cd.g_vec_new[c];
        p2.v[c] = cd.v_com[c] - I.mu1 * cd.g_vec_new[c];
    }
}

// ------------------------------------------------------------ collision_ntc.jl
inline uint32_t pair_code(const Orc& o, int s1, int s2) { return (uint32_t)(s1 * o.n_species + s2); }

// collide_2particles_vhs!, collision_ntc.jl:223-270.  pi_i / pi_k are physical
// slots (0-based) in particles_1 / particles_2 (re-fetched after a resize).
void collide_2particles_vhs(orc_stream* rng, CollisionData& cd, CollisionFactors& cf, const Interaction& I,
                            Orc& o, int64_t phys_i, int64_t phys_k, int s1, int s2, int64_t cell, double dw_tol)
{
    ParticleVector& P1 = o.pv[s1];
    ParticleVector& P2 = o.pv[s2];
    double wi = P1.particles[phys_i].w, wk = P2.particles[phys_k].w;
    double sigma = sigma_vhs(I, cd.g);
    double sgw = sigma * cd.g * std::max(wi, wk);
    cf.sigma_g_w_max = std::max(sgw, cf.sigma_g_w_max);
    if (orc_stream_uniform(rng) < sgw / cf.sigma_g_w_max) {
        cf.n_coll_performed += 1;
        compute_com(cd, I, P1.particles[phys_i], P2.particles[phys_k]);
        if (std::fabs(wi - wk) < dw_tol) {
            cf.n_eq_w_coll_performed += 1;
        } else if (wi > wk) {
            if (P1.length() <= o.n_total[s1]) pv_resize(P1, P1.length() + DELTA_PARTICLES);
            update_buffer_index_new_particle(o, cell, s1);
            double dw = wi - wk;
            Particle& pa_i = P1.particles[phys_i];
            pa_i.w = wk;
            Particle& np_ = P1.at(o.n_total[s1]);
            np_.w = dw;
            for (int c = 0; c < 3; ++c) {
                np_.v[c] = pa_i.v[c];
                np_.x[c] = pa_i.x[c];
            }
        } else {
            if (P2.length() <= o.n_total[s2]) pv_resize(P2, P2.length() + DELTA_PARTICLES);
            update_buffer_index_new_particle(o, cell, s2);
            double dw = wk - wi;
            Particle& pa_k = P2.particles[phys_k];
            pa_k.w = wi;
            Particle& np_ = P2.at(o.n_total[s2]);
            np_.w = dw;
            for (int c = 0; c < 3; ++c) {
                np_.v[c] = pa_k.v[c];
                np_.x[c] = pa_k.x[c];
            }
        }
        scatter_vhs(rng, cd, I, o.pv[s1].particles[phys_i], o.pv[s2].particles[phys_k]);
    }
}

// collide_2particles_vhs_equal_weight!, collision_ntc.jl:294-309
void collide_2particles_vhs_equal_weight(orc_stream* rng, CollisionData& cd, CollisionFactors& cf,
                                         const Interaction& I, Particle& pa_i, Particle& pa_k)
{
    double sigma = sigma_vhs(I, cd.g);
    double sgw = sigma * cd.g * std::max(pa_i.w, pa_k.w);
    cf.sigma_g_w_max = std::max(sgw, cf.sigma_g_w_max);
    if (orc_stream_uniform(rng) < sgw / cf.sigma_g_w_max) {
        cf.n_coll_performed += 1;
        cf.n_eq_w_coll_performed += 1;
        compute_com(cd, I, pa_i, pa_k);
        scatter_vhs(rng, cd, I, pa_i, pa_k);
    }
}

const double EPS = 2.220446049250313e-16;        // Julia eps()

// ntc! (single species, collision_ntc.jl:338-380) and ntc_equal_weight!
// (collision_ntc.jl:479-521); the candidate loop is identical, only the
// collide routine differs.
void ntc_single(Orc& o, int s, int64_t cell, double dt, double V, uint64_t seed, uint64_t step, double dw_tol,
                bool equal_weight)
{
    CollisionFactors& cf = o.cfa(s, s, cell);
    const uint32_t pc = pair_code(o, s, s);
    const uint32_t rc = (uint32_t)(cell - 1 + o.cell_offset);
    int64_t np = o.pi(cell, s).n_local;
    cf.n1 = np;
    cf.n2 = np;
    orc_stream r0 = orc_stream_make(seed, ORC_TAG_NCOLL, pc, step, rc, 0);
    double n_coll_float = 0.5 * dt * (double)np * (double)(np - 1) * cf.sigma_g_w_max / V + orc_stream_uniform(&r0);
    int64_t n_coll_int = (int64_t)std::floor(n_coll_float);
    cf.n_coll = n_coll_int;
    cf.n_coll_performed = 0;
    cf.n_eq_w_coll_performed = 0;
    const Interaction& I = o.inter[s + o.n_species * s];
    CollisionData cd;
    for (int64_t j = 0; j < n_coll_int; ++j) {
        orc_stream rng = orc_stream_make(seed, ORC_TAG_CAND, pc, step, rc, (uint32_t)j);
        int64_t nl = o.pi(cell, s).n_local;
        int64_t i = (int64_t)std::floor(orc_stream_uniform(&rng) * (double)nl);
        int64_t k = (int64_t)std::floor(orc_stream_uniform(&rng) * (double)nl);
        while (i == k) k = (int64_t)std::floor(orc_stream_uniform(&rng) * (double)nl);
        i = map_cont_index(o.pi(cell, s), i);
        k = map_cont_index(o.pi(cell, s), k);
        int64_t phys_i = o.pv[s].index[i - 1] - 1;
        int64_t phys_k = o.pv[s].index[k - 1] - 1;
        compute_g(cd, o.pv[s].particles[phys_i], o.pv[s].particles[phys_k]);
        if (cd.g > EPS) {
            if (equal_weight)
                collide_2particles_vhs_equal_weight(&rng, cd, cf, I, o.pv[s].particles[phys_i],
                                                    o.pv[s].particles[phys_k]);
            else
                collide_2particles_vhs(&rng, cd, cf, I, o, phys_i, phys_k, s, s, cell, dw_tol);
        }
    }
}

// ntc! two species (collision_ntc.jl:412-453) and ntc_equal_weight! two
// species (collision_ntc.jl:554-595).
void ntc_two(Orc& o, int s1, int s2, int64_t cell, double dt, double V, uint64_t seed, uint64_t step, double dw_tol,
             bool equal_weight)
{
    CollisionFactors& cf = o.cfa(s1, s2, cell);
    const uint32_t pc = pair_code(o, s1, s2);
    const uint32_t rc = (uint32_t)(cell - 1 + o.cell_offset);
    int64_t np1 = o.pi(cell, s1).n_local, np2 = o.pi(cell, s2).n_local;
    cf.n1 = np1;
    cf.n2 = np2;
    orc_stream r0 = orc_stream_make(seed, ORC_TAG_NCOLL, pc, step, rc, 0);
    double n_coll_float = dt * (double)np1 * (double)np2 * cf.sigma_g_w_max / V + orc_stream_uniform(&r0);
    int64_t n_coll_int = (int64_t)std::floor(n_coll_float);
    cf.n_coll = n_coll_int;
    cf.n_coll_performed = 0;
    cf.n_eq_w_coll_performed = 0;
    const Interaction& I = o.inter[s1 + o.n_species * s2];
    CollisionData cd;
    for (int64_t j = 0; j < n_coll_int; ++j) {
        orc_stream rng = orc_stream_make(seed, ORC_TAG_CAND, pc, step, rc, (uint32_t)j);
        int64_t i = (int64_t)std::floor(orc_stream_uniform(&rng) * (double)o.pi(cell, s1).n_local);
        int64_t k = (int64_t)std::floor(orc_stream_uniform(&rng) * (double)o.pi(cell, s2).n_local);
        i = map_cont_index(o.pi(cell, s1), i);
        k = map_cont_index(o.pi(cell, s2), k);
        int64_t phys_i = o.pv[s1].index[i - 1] - 1;
        int64_t phys_k = o.pv[s2].index[k - 1] - 1;
        compute_g(cd, o.pv[s1].particles[phys_i], o.pv[s2].particles[phys_k]);
        if (cd.g > EPS) {
            if (equal_weight)
                collide_2particles_vhs_equal_weight(&rng, cd, cf, I, o.pv[s1].particles[phys_i],
                                                    o.pv[s2].particles[phys_k]);
            else
                collide_2particles_vhs(&rng, cd, cf, I, o, phys_i, phys_k, s1, s2, cell, dw_tol);
        }
    }
}

// ------------------------------------------------------------ collision_swpm.jl
// swpm! (collision_swpm.jl:201-288) with compute_n_coll_single_species
// (:170-173).  The (sigma g)_max estimate lives in the pair's
// CollisionFactors (sigma_g_w_max field).  Draws come from the NTC streams:
// U for n_coll, then per candidate U_i, U_k, retries of U_k, U_acc (g > eps),
// U_phi, U_theta (accepted).  The reference checks the storage size once per
// accepted collision and then appends two particles; here each append checks.
void swpm_cell(Orc& o, int s, int64_t cell, double G, double dt, double V, uint64_t seed, uint64_t step)
{
    CollisionFactors& cf = o.cfa(s, s, cell);
    const uint32_t pc = pair_code(o, s, s);
    const uint32_t rc = (uint32_t)(cell - 1 + o.cell_offset);
    ParticleVector& P = o.pv[s];
    double w_max = 0.0;
    {
        const ParticleIndexer& p = o.pi(cell, s);
        for (int64_t i = p.start1; i <= p.end1; ++i) w_max = std::max(w_max, P.at(i).w);
        if (p.n_group2 > 0)
            for (int64_t i = p.start2; i <= p.end2; ++i) w_max = std::max(w_max, P.at(i).w);
    }
    const double wtf = 1.0 / (1.0 + G);
    const double inv_w_max = 1.0 / w_max;
    const int64_t np = o.pi(cell, s).n_local;
    cf.n1 = np;
    cf.n2 = np;
    orc_stream r0 = orc_stream_make(seed, ORC_TAG_NCOLL, pc, step, rc, 0);
    const double n_coll_float =
        0.5 * dt * (double)np * (double)(np - 1) * cf.sigma_g_w_max * w_max * (G + 1.0) / V + orc_stream_uniform(&r0);
    const int64_t n_coll_int = (int64_t)std::floor(n_coll_float);
    cf.n_coll = n_coll_int;
    cf.n_coll_performed = 0;
    const Interaction& I = o.inter[s + o.n_species * s];
    CollisionData cd;
    for (int64_t j = 0; j < n_coll_int; ++j) {
        orc_stream rng = orc_stream_make(seed, ORC_TAG_CAND, pc, step, rc, (uint32_t)j);
        const int64_t nl = o.pi(cell, s).n_local;
        int64_t i = (int64_t)std::floor(orc_stream_uniform(&rng) * (double)nl);
        int64_t k = (int64_t)std::floor(orc_stream_uniform(&rng) * (double)nl);
        while (i == k) k = (int64_t)std::floor(orc_stream_uniform(&rng) * (double)nl);
        i = map_cont_index(o.pi(cell, s), i);
        k = map_cont_index(o.pi(cell, s), k);
        const int64_t phys_i = P.index[i - 1] - 1;
        const int64_t phys_k = P.index[k - 1] - 1;
        compute_g(cd, P.particles[phys_i], P.particles[phys_k]);
        if (cd.g > EPS) {
            const double sigma = sigma_vhs(I, cd.g);
            const double sigma_g = sigma * cd.g;
            cf.sigma_g_w_max = std::max(sigma_g, cf.sigma_g_w_max);
            const double wm = std::max(P.particles[phys_i].w, P.particles[phys_k].w);
            if (orc_stream_uniform(&rng) < sigma_g * wm * inv_w_max / cf.sigma_g_w_max) {
                cf.n_coll_performed += 1;
                compute_com(cd, I, P.particles[phys_i], P.particles[phys_k]);
                const double dw = std::min(P.particles[phys_i].w, P.particles[phys_k].w) * wtf;
                P.particles[phys_i].w -= dw;
                P.particles[phys_k].w -= dw;
                for (int q = 0; q < 2; ++q) {
                    if (P.length() <= o.n_total[s]) pv_resize(P, P.length() + DELTA_PARTICLES);
                    update_buffer_index_new_particle(o, cell, s);
                    Particle& src = P.particles[q == 0 ? phys_i : phys_k];
                    Particle& dst = P.at(o.n_total[s]);
                    dst.w = dw;
                    for (int c = 0; c < 3; ++c) {
                        dst.v[c] = src.v[c];
                        dst.x[c] = src.x[c];
                    }
                }
                scatter_vhs(&rng, cd, I, P.at(o.n_total[s] - 1), P.at(o.n_total[s]));
            }
        }
    }
}

// ----------------------------------------------------------- physical_props.jl
struct PropsOut {
    double* lpa;
    double* np;       // [cell + n_cells * s]
    double* n;
    double* v;        // [c + 3 * (cell + n_cells * s)]
    double* T;
    double* moments;  // [m + n_mom * (cell + n_cells * s)]
};

// compute_props! (physical_props.jl:104-154) when n_moments == 0, and
// compute_props_with_total_moments! (physical_props.jl:168-245) otherwise.
void compute_props(Orc& o, const int32_t* powers, int32_t n_mom, double Tref, PropsOut out, bool with_moments,
                   int nthreads)
{
    const int64_t nc = o.n_cells;
    for (int s = 0; s < o.n_species; ++s) {
        double mass = o.mass[s];
        double moment_factor = 0.0, moment_vref = 0.0;
        if (with_moments && n_mom > 0) {
            moment_factor = 4.0 * PI * std::pow(mass / (twopi * k_B * Tref), 1.5) * 0.5;
            moment_vref = std::pow(mass / (2.0 * k_B * Tref), 0.5);
        }
        ParticleVector& pv = o.pv[s];
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 64) if (nthreads > 1)
        for (int64_t cell = 1; cell <= nc; ++cell) {
            ParticleIndexer p = o.pi(cell, s);
            int64_t np = 0;
            double n = 0.0, E = 0.0, T = 0.0;
            double v[3] = {0, 0, 0};
            std::vector<double> mom(with_moments ? n_mom : 0, 0.0);
            auto acc1 = [&](int64_t i) {
                const Particle& q = pv.at(i);
                n += q.w;
                for (int c = 0; c < 3; ++c) v[c] = v[c] + q.v[c] * q.w;
                np += 1;
            };
            for (int64_t i = p.start1; i <= p.end1; ++i) acc1(i);
            if (p.n_group2 > 0)
                for (int64_t i = p.start2; i <= p.end2; ++i) acc1(i);
            if (n > 0.0) {
                for (int c = 0; c < 3; ++c) v[c] = v[c] / n;
                auto acc2 = [&](int64_t i) {
                    const Particle& q = pv.at(i);
                    double d0 = q.v[0] - v[0], d1 = q.v[1] - v[1], d2 = q.v[2] - v[2];
                    if (with_moments) {
                        double normv = std::sqrt((d0 * d0 + d1 * d1) + d2 * d2);
                        E = std::fma(q.w, normv * normv, E);
                        for (int m = 0; m < n_mom; ++m)
                            mom[m] = std::fma(q.w, std::pow(normv, (double)powers[m]), mom[m]);
                    } else {
                        E = std::fma(q.w, (d0 * d0 + d1 * d1) + d2 * d2, E);
                    }
                };
                for (int64_t i = p.start1; i <= p.end1; ++i) acc2(i);
                if (p.n_group2 > 0)
                    for (int64_t i = p.start2; i <= p.end2; ++i) acc2(i);
                E *= 0.5 * mass / (n * k_B);
                T = (2.0 / 3.0) * E;
            }
            if (with_moments) {
                for (int m = 0; m < n_mom; ++m) {
                    double mm = (double)powers[m];
                    double scaling = moment_factor * std::pow(moment_vref, -(3.0 + mm)) * std::tgamma((3.0 + mm) / 2.0);
                    mom[m] /= (scaling * n);
                    out.moments[m + n_mom * ((cell - 1) + nc * s)] = mom[m];
                }
            }
            int64_t ix = (cell - 1) + nc * s;
            out.np[ix] = (double)np;
            out.n[ix] = n;
            for (int c = 0; c < 3; ++c) out.v[c + 3 * ix] = v[c];
            out.T[ix] = T;
        }
        if (out.lpa) out.lpa[s] = (double)pv.length();
    }
}

// compute_props_sorted! (physical_props.jl:317-354) and the grid / number
// density variant (physical_props.jl:393-433) when inv_V != nullptr.
void compute_props_sorted(Orc& o, PropsOut out, const double* inv_V, int nthreads)
{
    const int64_t nc = o.n_cells;
    for (int s = 0; s < o.n_species; ++s) {
        double mass = o.mass[s];
        ParticleVector& pv = o.pv[s];
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 64) if (nthreads > 1)
        for (int64_t cell = 1; cell <= nc; ++cell) {
            ParticleIndexer p = o.pi(cell, s);
            double n = 0.0, E = 0.0, T = 0.0;
            double v[3] = {0, 0, 0};
            int64_t s1 = p.start1, e1 = p.end1;
            for (int64_t i = s1; i <= e1; ++i) {
                const Particle& q = pv.at(i);
                n += q.w;
                for (int c = 0; c < 3; ++c) v[c] = v[c] + q.v[c] * q.w;
            }
            double np = e1 >= s1 ? (double)(e1 - s1) + 1.0 : 0.0;
            if (n > 0.0) {
                for (int c = 0; c < 3; ++c) v[c] = v[c] / n;
                for (int64_t i = s1; i <= e1; ++i) {
                    const Particle& q = pv.at(i);
                    double d0 = q.v[0] - v[0], d1 = q.v[1] - v[1], d2 = q.v[2] - v[2];
                    E = std::fma(q.w, (d0 * d0 + d1 * d1) + d2 * d2, E);
                }
                E *= 0.5 * mass / (n * k_B);
                T = (2.0 / 3.0) * E;
            }
            int64_t ix = (cell - 1) + nc * s;
            out.np[ix] = np;
            out.n[ix] = inv_V ? n * inv_V[cell - 1] : n;
            for (int c = 0; c < 3; ++c) out.v[c + 3 * ix] = v[c];
            out.T[ix] = T;
        }
    }
}

// ------------------------------------------------------ boundary_conditions.jl
struct Walls {                                   // MaxwellWalls1D, boundary_conditions.jl:29-53
    double T[2];
    double v[2][3];
    double acc[2];
    std::vector<double> vsq;                     // [wall + 2 * s]
};

inline void specular_reflection_x(Particle& p) { p.v[0] = -p.v[0]; }  // boundary_conditions.jl:63-65

inline void diffuse_reflection_x(orc_stream* rng, Particle& p, double vsq, double normal, const double* wv)
{   // boundary_conditions.jl:79-93
    double R = std::max(1e-50, orc_stream_uniform(rng));
    double v_normal = normal * std::sqrt(-vsq * std::log(R));
    R = std::max(1e-50, orc_stream_uniform(rng));
    double v_tang = std::sqrt(-vsq * std::log(R));
    R = twopi * orc_stream_uniform(rng);
    double v_tang1 = std::sin(R) * v_tang;
    double v_tang2 = std::cos(R) * v_tang;
    p.v[0] = v_normal + wv[0];
    p.v[1] = v_tang1 + wv[1];
    p.v[2] = v_tang2 + wv[2];
}

inline void reflect_particle_x(orc_stream* rng, Particle& p, double vsq, double normal, const double* wv, double acc)
{   // boundary_conditions.jl:108-121
    if (acc == 0.0) {
        specular_reflection_x(p);
    } else if (acc == 1.0) {
        diffuse_reflection_x(rng, p, vsq, normal, wv);
    } else {
        double R = orc_stream_uniform(rng);
        if (R < acc)
            diffuse_reflection_x(rng, p, vsq, normal, wv);
        else
            specular_reflection_x(p);
    }
}

// ----------------------------------------------------------- grid_uniform1D.jl
struct Grid1D {                                  // Grid1DUniform, grid_uniform1D.jl:49-86
    double L;
    int64_t n_cells;
    double dx, inv_dx, min_x, max_x;
};

Grid1D make_grid(double L, int64_t nx, double wall_offset)
{
    Grid1D g;
    g.L = L;
    g.n_cells = nx;
    g.dx = L / (double)nx;
    g.inv_dx = 1.0 / g.dx;
    g.min_x = g.dx * wall_offset;
    g.max_x = std::fma(-g.dx, wall_offset, L);   // @muladd: L - dx * wall_offset
    return g;
}

inline int64_t get_cell(const Grid1D& g, double x) { return (int64_t)std::floor(x * g.inv_dx) + 1; }  // :97-99

// ------------------------------------------------------------- convection_1D.jl
// SurfProps of a 1-D grid for one species (surface_props.jl:22-67):
// element 0 = left wall (normal +x), element 1 = right wall (normal -x), unit
// areas; per element np, flux_incident, flux_reflected, force[3],
// normal_pressure, shear_pressure[3], kinetic_energy_flux.
enum { SQ_NP, SQ_FIN, SQ_FREF, SQ_FX, SQ_FY, SQ_FZ, SQ_PN, SQ_SX, SQ_SY, SQ_SZ, SQ_KE, SQ_N };
struct Surf {
    double q[2][SQ_N] = {{0}};
};

inline double surf_normal_x(int e) { return e == 0 ? 1.0 : -1.0; }

// update_surface_incident! (surface_props.jl:78-101), sign +1, and
// update_surface_reflected! (:113-134), sign -1
void surf_update(double* q, int e, double w, const double* v, bool reflected)
{
    const double n[3] = {surf_normal_x(e), 0.0, 0.0};
    const double px = w * v[0], py = w * v[1], pz = w * v[2];
    const double pn = px * n[0] + py * n[1] + pz * n[2];
    const double sg = reflected ? -1.0 : 1.0;
    if (!reflected) {
        q[SQ_NP] += 1.0;
        q[SQ_FIN] += w;
    } else {
        q[SQ_FREF] -= w;
    }
    q[SQ_FX] += sg * px;
    q[SQ_FY] += sg * py;
    q[SQ_FZ] += sg * pz;
    q[SQ_PN] -= sg * pn;
    q[SQ_SX] += sg * (px - pn * n[0]);
    q[SQ_SY] += sg * (py - pn * n[1]);
    q[SQ_SZ] += sg * (pz - pn * n[2]);
    q[SQ_KE] += sg * (0.5 * (px * v[0] + py * v[1] + pz * v[2]));
}

// surface_props_scale! (surface_props.jl:149-166): all but np times mass / dt / area
void surf_scale(double* q, double mass, double dt, double inv_area)
{
    const double f = mass / dt * inv_area;
    for (int k = SQ_FIN; k < SQ_N; ++k) q[k] *= f;
}

void convect_single_particle(orc_stream* rng, const Grid1D& g, const Walls& W, Particle& p, int s, double dt,
                             Surf* surf = nullptr)
{   // convection_1D.jl:17-54 (with surf: :72-112)
    double t_rest = dt;
    double x_old = p.x[0];
    double x_new = std::fma(p.v[0], dt, p.x[0]);
    int hits = 0;
    while ((x_new >= g.L) || (x_new <= 0.0)) {
        if (hits++ >= ORC_MAX_WALL_HITS) break;
        int bc;
        double normal;
        if (x_new >= g.L) {
            t_rest -= std::fabs((g.L - x_old) / p.v[0]);
            bc = 1;
            normal = -1.0;
            x_old = g.L;
        } else {
            t_rest -= std::fabs(x_old / p.v[0]);
            bc = 0;
            normal = 1.0;
            x_old = 0.0;
        }
        if (surf) surf_update(surf->q[bc], bc, p.w, p.v, false);
        reflect_particle_x(rng, p, W.vsq[bc + 2 * s], normal, W.v[bc], W.acc[bc]);
        if (surf) surf_update(surf->q[bc], bc, p.w, p.v, true);
        x_new = std::fma(p.v[0], t_rest, x_old);
    }
    x_new = std::min(std::max(x_new, g.min_x), g.max_x);  // clamp
    p.x[0] = x_new;
}

// convect_particles! (convection_1D.jl:130-157) and
// convect_particles_and_compute_cell! (convection_1D.jl:225-255); with surf,
// convect_particles!(..., surf_props, dt) (:176-206), sequential so the
// surface sums keep the reference's order.  Each particle's stream is keyed
// on (cell, position j in the cell's logical list).
void convect_particles(Orc& o, int s, const Grid1D& g, const Walls& W, double dt, uint64_t seed, uint64_t step,
                       bool compute_cell, int nthreads, Surf* surf = nullptr)
{
    ParticleVector& pv = o.pv[s];
    const int64_t nc = o.n_cells;
    if (surf) nthreads = 1;
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 64) if (nthreads > 1)
    for (int64_t cell = 1; cell <= nc; ++cell) {
        ParticleIndexer p = o.pi(cell, s);
        int64_t j = 0;
        auto one = [&](int64_t i) {
            orc_stream rng = orc_stream_make(seed, ORC_TAG_CONVECT, (uint32_t)s, step, (uint32_t)(cell - 1 + o.cell_offset),
                                              (uint32_t)j);
            ++j;
            convect_single_particle(&rng, g, W, pv.at(i), s, dt, surf);
            if (compute_cell) pv.cell[i - 1] = get_cell(g, pv.at(i).x[0]);
        };
        for (int64_t i = p.start1; i <= p.end1; ++i) one(i);
        if (p.n_group2 > 0)
            for (int64_t i = p.start2; i <= p.end2; ++i) one(i);
    }
    if (surf)
        for (int e = 0; e < 2; ++e) surf_scale(surf->q[e], o.mass[s], dt, 1.0);
}

// --------------------------------------------------------------- grid_sorting.jl
// sort_particles!(gridsort, grid, particles, pia, species) (grid_sorting.jl:58-113)
// when `grid` is given, sort_particles!(gridsort, particles, pia, species)
// (grid_sorting.jl:128-182) otherwise.
void sort_particles(Orc& o, int s, const Grid1D* g)
{
    ParticleVector& pv = o.pv[s];
    int64_t n_tot = o.n_total[s];
    const int64_t nc = o.n_cells;
    std::vector<int64_t> cell_counts(nc + 1, 0);
    std::vector<int64_t> sorted(std::max<int64_t>(n_tot, 1));
    if (!o.contiguous[s]) squash_pia(o, s);
    for (int64_t i = 1; i <= n_tot; ++i) {
        if (g) {
            int64_t newcell = get_cell(*g, pv.at(i).x[0]);
            pv.cell[i - 1] = newcell;
            cell_counts[newcell] += 1;
        } else {
            cell_counts[pv.cell[i - 1]] += 1;
        }
    }
    for (int64_t cell = 1; cell <= nc; ++cell) {
        cell_counts[cell] = cell_counts[cell] + cell_counts[cell - 1];
        int64_t cell_start = cell_counts[cell - 1] + 1;
        int64_t cell_np = cell_counts[cell] - cell_counts[cell - 1];
        int64_t cell_end = cell_counts[cell];
        ParticleIndexer& p = o.pi(cell, s);
        p.start2 = 0;
        p.end2 = -1;
        p.n_group2 = 0;
        if (cell_np > 0) {
            p.start1 = cell_start;
            p.end1 = cell_end;
        } else {
            p.start1 = 0;
            p.end1 = -1;
        }
        p.n_group1 = cell_np;
        p.n_local = cell_np;
    }
    for (int64_t i = n_tot; i >= 1; --i) {
        int64_t cur = pv.cell[i - 1];
        sorted[cell_counts[cur] - 1] = pv.index[i - 1];
        cell_counts[cur] -= 1;
    }
    for (int64_t i = 1; i <= n_tot; ++i) pv.index[i - 1] = sorted[i - 1];
    o.contiguous[s] = 1;
}

// --------------------------------------------------------- merging_octree_N2.jl
enum { SPLIT_MID = 1, SPLIT_MEAN = 2, SPLIT_MEDIAN = 3 };               // :12
enum { INIT_MINMAX = 1, INIT_MINMAX_SYM = 2, INIT_C = 3 };               // :24
enum { BOUNDS_INHERIT = 1, BOUNDS_RECOMPUTE = 2 };                       // :34

struct OctreeCell {                              // :49-59
    int64_t np = 0;
    double w = 0.0;
    double vmin[3] = {0, 0, 0}, vmax[3] = {0, 0, 0};
    int64_t depth = 0;
    bool can_be_refined = true;
};

struct OctreeFullCell {                          // :82-96
    double v_mean[3] = {0, 0, 0}, v_std_sq[3] = {0, 0, 0}, x_mean[3] = {0, 0, 0}, x_std_sq[3] = {0, 0, 0};
    int64_t pi1 = 0, pi2 = 0;
    double w1 = 0, w2 = 0, v1[3] = {0, 0, 0}, v2[3] = {0, 0, 0}, x1[3] = {0, 0, 0}, x2[3] = {0, 0, 0};
};

struct Octree {                                  // OctreeN2Merge, :131-179
    int64_t max_Nbins, Nbins = 0;
    std::vector<OctreeCell> bins;
    std::vector<OctreeFullCell> full_bins;
    int64_t n_particles = 0;
    std::vector<int64_t> bin_start, bin_end;     // 1-based positions into pis
    std::vector<int64_t> pis;                    // particle_indexes_sorted (ParticleVector positions)
    std::vector<int64_t> octants, sort_out;
    int64_t counter[8], nonempty_counter[8], nonempty_bins[8];
    double ndens_counter[8];
    int bounds_mode, split, init_bounds;
    double vel_middle[3] = {0, 0, 0}, vmin_parent[3], vmax_parent[3];
    int64_t max_depth, total_post_merge_np = 0;
};

Octree* octree_new(int split, int init_bounds, int bounds_mode, int64_t max_Nbins, int64_t max_depth)
{   // OctreeN2Merge(...), :235-246
    Octree* oc = new Octree();
    oc->max_Nbins = max_Nbins;
    oc->bins.resize(max_Nbins);
    oc->full_bins.resize(max_Nbins);
    oc->bin_start.assign(max_Nbins, 0);
    oc->bin_end.assign(max_Nbins, 0);
    oc->pis.assign(8192, 0);
    oc->octants.assign(8192, 0);
    oc->sort_out.assign(8192, 0);
    oc->split = split;
    oc->init_bounds = init_bounds;
    oc->bounds_mode = bounds_mode;
    oc->max_depth = max_depth;
    return oc;
}

void resize_octree_buffers(Octree& oc, int64_t n)  // :270-280
{
    if ((int64_t)oc.pis.size() < n) oc.pis.resize(n + DELTA_PARTICLES);
    if ((int64_t)oc.octants.size() < n) oc.octants.resize(n + DELTA_PARTICLES);
    if ((int64_t)oc.sort_out.size() < n) oc.sort_out.resize(n + DELTA_PARTICLES);
}

inline int compute_octant(const double* v, const double* mid)  // :304-316
{
    int oct = 1;
    if (v[0] > mid[0]) oct += 1;
    if (v[1] > mid[1]) oct += 2;
    if (v[2] > mid[2]) oct += 4;
    return oct;
}

void bin_bounds_inherit(Octree& oc, int64_t bin_id, const double* pmin, const double* pmax, const double* mid,
                        int64_t octant)       // :341-367
{
    OctreeCell& b = oc.bins[bin_id - 1];
    int64_t o = octant - 1;
    for (int c = 0; c < 3; ++c) {
        bool upper = (o >> c) & 1;
        b.vmin[c] = upper ? mid[c] : pmin[c];
        b.vmax[c] = upper ? pmax[c] : mid[c];
    }
}

void bin_bounds_recompute(Octree& oc, int64_t bin_id, int64_t bs, int64_t be, ParticleVector& pv)  // :382-418
{
    double mn[3] = {9299792458.0, 9299792458.0, 9299792458.0};
    double mx[3] = {-9299792458.0, -9299792458.0, -9299792458.0};
    OctreeCell& b = oc.bins[bin_id - 1];
    for (int64_t i = bs; i <= be; ++i) {
        const Particle& q = pv.at(oc.pis[i - 1]);
        for (int c = 0; c < 3; ++c) {
            if (q.v[c] < mn[c]) mn[c] = q.v[c];
            if (q.v[c] > mx[c]) mx[c] = q.v[c];
        }
        for (int c = 0; c < 3; ++c) {
            b.vmin[c] = mn[c];
            b.vmax[c] = mx[c];
        }
    }
}

void compute_v_mean(Octree& oc, int64_t bs, int64_t be, ParticleVector& pv)  // :431-439
{
    double n_tot = 0.0;
    for (int64_t i = bs; i <= be; ++i) {
        const Particle& q = pv.at(oc.pis[i - 1]);
        n_tot += q.w;
        for (int c = 0; c < 3; ++c) oc.vel_middle[c] = oc.vel_middle[c] + q.w * q.v[c];
    }
    for (int c = 0; c < 3; ++c) oc.vel_middle[c] = oc.vel_middle[c] / n_tot;
}

inline int64_t get_new_bin_id(int64_t i, int64_t bin_id, int64_t Nbins) { return i == 1 ? bin_id : Nbins + i - 1; }

inline int64_t get_bin_post_merge_np(const Octree& oc, int64_t bin_id)  // :715-720
{
    int64_t np = oc.bins[bin_id - 1].np;
    return np >= 2 ? 2 : np;
}

void split_bin(Octree& oc, int64_t bin_id, ParticleVector& pv)  // :503-633
{
    int64_t n_nonempty = 0;
    for (int i = 0; i < 8; ++i) {
        oc.counter[i] = 0;
        oc.ndens_counter[i] = 0.0;
        oc.nonempty_bins[i] = 0;
        oc.nonempty_counter[i] = 0;
    }
    int64_t current_depth = oc.bins[bin_id - 1].depth;
    int64_t bs = oc.bin_start[bin_id - 1];
    int64_t be = oc.bin_end[bin_id - 1];
    if (oc.bounds_mode == BOUNDS_RECOMPUTE) bin_bounds_recompute(oc, bin_id, bs, be, pv);
    if (oc.split == SPLIT_MID) {
        for (int c = 0; c < 3; ++c)
            oc.vel_middle[c] = 0.5 * (oc.bins[bin_id - 1].vmin[c] + oc.bins[bin_id - 1].vmax[c]);
    } else if (oc.split == SPLIT_MEAN) {
        compute_v_mean(oc, bs, be, pv);
    }
    for (int64_t i = bs; i <= be; ++i) {
        int64_t pin = oc.pis[i - 1];
        int oct = compute_octant(pv.at(pin).v, oc.vel_middle);
        oc.counter[oct - 1] += 1;
        oc.octants[i - bs] = oct;
        oc.ndens_counter[oct - 1] += pv.at(pin).w;
    }
    int64_t n_eb = 0;
    if (oc.counter[0] > 0) {
        n_nonempty += 1;
        n_eb += 1;
        oc.nonempty_counter[n_eb - 1] = oc.counter[0];
        oc.nonempty_bins[n_eb - 1] = 1;
    }
    for (int i = 2; i <= 8; ++i) {
        if (oc.counter[i - 1] > 0) {
            n_nonempty += 1;
            n_eb += 1;
            oc.nonempty_counter[n_eb - 1] = oc.counter[i - 1];
            oc.nonempty_bins[n_eb - 1] = i;
        }
        oc.counter[i - 1] += oc.counter[i - 2];
    }
    oc.bin_end[bin_id - 1] = oc.bin_start[bin_id - 1] + oc.nonempty_counter[0] - 1;
    for (int64_t i = 2; i <= n_nonempty; ++i) {
        int64_t bi = get_new_bin_id(i, bin_id, oc.Nbins);
        int64_t bim1 = get_new_bin_id(i - 1, bin_id, oc.Nbins);
        oc.bin_start[bi - 1] = oc.bin_end[bim1 - 1] + 1;
        oc.bin_end[bi - 1] = oc.bin_start[bi - 1] + oc.nonempty_counter[i - 1] - 1;
    }
    oc.total_post_merge_np -= 2;
    if (oc.bounds_mode == BOUNDS_INHERIT) {
        for (int c = 0; c < 3; ++c) {
            oc.vmin_parent[c] = oc.bins[bin_id - 1].vmin[c];
            oc.vmax_parent[c] = oc.bins[bin_id - 1].vmax[c];
        }
    }
    for (int64_t i = 1; i <= n_nonempty; ++i) {
        int64_t bi = get_new_bin_id(i, bin_id, oc.Nbins);
        if (oc.bounds_mode == BOUNDS_INHERIT)
            bin_bounds_inherit(oc, bi, oc.vmin_parent, oc.vmax_parent, oc.vel_middle, oc.nonempty_bins[i - 1]);
        OctreeCell& b = oc.bins[bi - 1];
        b.np = oc.nonempty_counter[i - 1];
        b.w = oc.ndens_counter[oc.nonempty_bins[i - 1] - 1];
        b.depth = current_depth + 1;
        oc.total_post_merge_np += get_bin_post_merge_np(oc, bi);
        b.can_be_refined = (b.np > 2) && (b.depth < oc.max_depth);
    }
    for (int64_t i = bs; i <= be; ++i) {
        int64_t pin = oc.pis[i - 1];
        int64_t j = oc.octants[i - bs];
        oc.sort_out[oc.counter[j - 1] - 1] = pin;
        oc.counter[j - 1] -= 1;
    }
    for (int64_t i = bs; i <= be; ++i) oc.pis[i - 1] = oc.sort_out[i - bs];
    oc.Nbins += n_nonempty - 1;
}

void compute_bin_props(Octree& oc, int64_t bin_id, ParticleVector& pv)  // :646-700
{
    int64_t bs = oc.bin_start[bin_id - 1];
    int64_t be = oc.bin_end[bin_id - 1];
    OctreeCell& b = oc.bins[bin_id - 1];
    OctreeFullCell& f = oc.full_bins[bin_id - 1];
    if (b.w == 0) {
        b.np = 0;
        return;
    }
    if (b.np == 1) {
        f.pi1 = oc.pis[bs - 1];
    } else if (b.np >= 2) {
        f.pi1 = oc.pis[bs - 1];
        f.pi2 = oc.pis[bs];
    }
    if (b.np <= 2) return;
    double vm[3] = {0, 0, 0}, vs[3] = {0, 0, 0}, xm[3] = {0, 0, 0}, xs[3] = {0, 0, 0};
    double inv_w = 1.0 / b.w;
    for (int64_t i = bs; i <= be; ++i) {
        const Particle& q = pv.at(oc.pis[i - 1]);
        for (int c = 0; c < 3; ++c) {
            vm[c] = vm[c] + q.w * q.v[c];
            xm[c] = xm[c] + q.w * q.x[c];
        }
    }
    for (int c = 0; c < 3; ++c) {
        vm[c] = vm[c] * inv_w;
        xm[c] = xm[c] * inv_w;
    }
    for (int64_t i = bs; i <= be; ++i) {
        const Particle& q = pv.at(oc.pis[i - 1]);
        for (int c = 0; c < 3; ++c) {
            double dv = q.v[c] - vm[c], dx = q.x[c] - xm[c];
            vs[c] = vs[c] + q.w * (dv * dv);
            xs[c] = xs[c] + q.w * (dx * dx);
        }
    }
    for (int c = 0; c < 3; ++c) {
        f.v_mean[c] = vm[c];
        f.v_std_sq[c] = vs[c] * inv_w;
        f.x_mean[c] = xm[c];
        f.x_std_sq[c] = xs[c] * inv_w;
    }
}

void init_octree(Octree& oc, Orc& o, int s, int64_t cell)  // :947-984
{
    ParticleIndexer p = o.pi(cell, s);
    ParticleVector& pv = o.pv[s];
    oc.Nbins = 1;
    for (int64_t i = 0; i < p.n_group1; ++i) oc.pis[i] = p.start1 + i;
    if (p.n_group2 > 0)
        for (int64_t i = 0; i < p.n_local - p.n_group1; ++i) oc.pis[p.n_group1 + i] = p.start2 + i;
    oc.n_particles = p.n_local;
    OctreeCell& b = oc.bins[0];
    b.depth = 0;
    oc.bin_start[0] = 1;
    oc.bin_end[0] = oc.n_particles;
    b.np = oc.n_particles;
    b.w = 1e50;
    oc.total_post_merge_np = get_bin_post_merge_np(oc, 1);
    b.can_be_refined = (b.np > 2) && (oc.max_depth > 0);
    if (oc.init_bounds == INIT_C) {
        for (int c = 0; c < 3; ++c) {
            b.vmin[c] = -299792458.0;
            b.vmax[c] = 299792458.0;
        }
    } else {
        bin_bounds_recompute(oc, 1, 1, oc.n_particles, pv);
        if (oc.init_bounds == INIT_MINMAX_SYM) {
            for (int c = 0; c < 3; ++c) {
                double m = std::max(std::fabs(b.vmin[c]), std::fabs(b.vmax[c]));
                b.vmin[c] = -m;
                b.vmax[c] = m;
            }
        }
    }
}

void compute_octree(Octree& oc, ParticleVector& pv, int64_t target_np)  // :998-1039
{
    while (true) {
        int64_t refine_id = -1;
        double max_w = -1.0;
        for (int64_t bin_id = 1; bin_id <= oc.Nbins; ++bin_id) {
            const OctreeCell& b = oc.bins[bin_id - 1];
            if ((b.w > max_w) && b.can_be_refined) {
                max_w = b.w;
                refine_id = bin_id;
            }
        }
        if (refine_id == -1) break;
        if (oc.total_post_merge_np + 14 > target_np) break;
        split_bin(oc, refine_id, pv);
        if (oc.Nbins + 7 > oc.max_Nbins) break;
    }
    if (oc.Nbins == 1) {
        oc.bins[0].w = 0.0;
        for (int64_t ii = 1; ii <= oc.n_particles; ++ii) oc.bins[0].w += pv.at(oc.pis[ii - 1]).w;
    }
    for (int64_t bin_id = 1; bin_id <= oc.Nbins; ++bin_id) compute_bin_props(oc, bin_id, pv);
}

inline double direction_sign(orc_stream* rng) { return orc_stream_uniform(rng) < 0.5 ? -1.0 : 1.0; }

// compute_new_particles!, :736-813 (no grid) and :830-933 (1D clamp)
void compute_new_particles(orc_stream* rng, Octree& oc, Orc& o, int s, int64_t cell, const Grid1D* g)
{
    ParticleVector& pv = o.pv[s];
    for (int64_t bin_id = 1; bin_id <= oc.Nbins; ++bin_id) {
        OctreeCell& b = oc.bins[bin_id - 1];
        OctreeFullCell& f = oc.full_bins[bin_id - 1];
        int64_t loc_np = b.np;
        if (loc_np > 2) {
            f.w1 = 0.5 * b.w;
            f.w2 = f.w1;
            for (int c = 0; c < 3; ++c) {
                f.v_std_sq[c] = std::sqrt(f.v_std_sq[c]);
                f.x_std_sq[c] = std::sqrt(f.x_std_sq[c]);
            }
            double d[3];
            for (int c = 0; c < 3; ++c) d[c] = direction_sign(rng);
            for (int c = 0; c < 3; ++c) {
                f.v1[c] = f.v_mean[c] + d[c] * f.v_std_sq[c];
                f.v2[c] = f.v_mean[c] - d[c] * f.v_std_sq[c];
            }
            for (int c = 0; c < 3; ++c) d[c] = direction_sign(rng);
            for (int c = 0; c < 3; ++c) {
                f.x1[c] = f.x_mean[c] + d[c] * f.x_std_sq[c];
                f.x2[c] = f.x_mean[c] - d[c] * f.x_std_sq[c];
            }
        } else if (loc_np == 2) {
            const Particle& q1 = pv.at(f.pi1);
            f.w1 = q1.w;
            std::memcpy(f.v1, q1.v, sizeof f.v1);
            std::memcpy(f.x1, q1.x, sizeof f.x1);
            const Particle& q2 = pv.at(f.pi2);
            f.w2 = q2.w;
            std::memcpy(f.v2, q2.v, sizeof f.v2);
            std::memcpy(f.x2, q2.x, sizeof f.x2);
        } else if (loc_np == 1) {
            const Particle& q1 = pv.at(f.pi1);
            f.w1 = q1.w;
            std::memcpy(f.v1, q1.v, sizeof f.v1);
            std::memcpy(f.x1, q1.x, sizeof f.x1);
        }
    }
    int64_t cur = 0;
    ParticleIndexer p = o.pi(cell, s);
    auto put = [&](double w, const double* v, const double* x, bool clampx) {
        int64_t i = map_cont_index(p, cur);
        cur += 1;
        Particle& q = pv.at(i);
        q.w = w;
        std::memcpy(q.v, v, sizeof q.v);
        std::memcpy(q.x, x, sizeof q.x);
        if (clampx && g) {
            if (x[0] < g->min_x)
                q.x[0] = g->min_x;
            else if (x[0] > g->max_x)
                q.x[0] = g->max_x;
        }
    };
    for (int64_t bin_id = 1; bin_id <= oc.Nbins; ++bin_id) {
        const OctreeCell& b = oc.bins[bin_id - 1];
        const OctreeFullCell& f = oc.full_bins[bin_id - 1];
        if (b.np >= 2) {
            bool big = b.np > 2;
            put(f.w1, f.v1, f.x1, big);
            put(f.w2, f.v2, f.x2, big);
        } else if (b.np == 1) {
            put(f.w1, f.v1, f.x1, false);
        }
    }
    int64_t old_count = o.pi(cell, s).n_local;
    int64_t n_del = old_count - cur;
    if (!(cell == o.n_cells) || (n_del > o.pi(cell, s).n_group2)) o.contiguous[s] = 0;
    for (int64_t k = 0; k < n_del; ++k) delete_particle_end(o, cell, s);
}

void merge_octree_N2_based(Octree& oc, Orc& o, int s, int64_t cell, int64_t target, const Grid1D* g, uint64_t seed,
                           uint64_t step)     // :1060-1066 and :1088-1094
{
    orc_stream rng = orc_stream_make(seed, ORC_TAG_MERGE, (uint32_t)s, step, (uint32_t)(cell - 1 + o.cell_offset), 0);
    oc.Nbins = 0;
    resize_octree_buffers(oc, o.pi(cell, s).n_local);
    init_octree(oc, o, s, cell);
    compute_octree(oc, o.pv[s], target);
    compute_new_particles(&rng, oc, o, s, cell, g);
}

// ------------------------------------------------- distributions_and_sampling.jl
void sample_maxwellian_one(orc_stream* rng, Particle& q, double vscale, const double* v0)
{   // sample_maxwellian!, distributions_and_sampling.jl:432-443 (log(1-U), see header)
    double vn = std::sqrt(-std::log(1.0 - orc_stream_uniform(rng)));
    double vr = std::sqrt(-std::log(1.0 - orc_stream_uniform(rng)));
    double t1 = twopi * orc_stream_uniform(rng);
    double t2 = twopi * orc_stream_uniform(rng);
    double u[3] = {vn * std::cos(t1), vr * std::cos(t2), vr * std::sin(t2)};
    for (int c = 0; c < 3; ++c) q.v[c] = vscale * u[c] + v0[c];
}

void sample_bkw_one(orc_stream* rng, Particle& q, double vscale, const double* v0)
{   // sample_bkw!, distributions_and_sampling.jl:195-213; Chi(5) = norm of 5
    // standard normals (Box-Muller pairs), Theta = pi U, phi = 2 pi U.
    double z[6];
    for (int k = 0; k < 3; ++k) {
        double r = std::sqrt(-2.0 * std::log(1.0 - orc_stream_uniform(rng)));
        double a = twopi * orc_stream_uniform(rng);
        z[2 * k] = r * std::cos(a);
        z[2 * k + 1] = r * std::sin(a);
    }
    double vabs = std::sqrt(z[0] * z[0] + z[1] * z[1] + z[2] * z[2] + z[3] * z[3] + z[4] * z[4]);
    double th = orc_stream_uniform(rng) * PI;
    double ph = orc_stream_uniform(rng) * twopi;
    double st = std::sin(th);
    double u[3] = {vabs * st * std::cos(ph), vabs * st * std::sin(ph), vabs * std::cos(th)};
    for (int c = 0; c < 3; ++c) q.v[c] = vscale * u[c] + v0[c];
}

// sample_particles_equal_weight!(rng, particles, pia, cell, species, n, m, T,
// Fnum, box...; distribution), distributions_and_sampling.jl:477-509
void sample_particles_equal_weight(Orc& o, int s, int64_t cell, int64_t n, double T, double Fnum, const double* box,
                                   uint64_t seed, uint64_t step, int distribution, const double* v0)
{
    ParticleVector& pv = o.pv[s];
    int64_t start = o.n_total[s] + 1;
    ParticleIndexer& p = o.pi(cell, s);
    p.n_local = n;
    o.n_total[s] += n;
    p.start1 = start;
    p.end1 = start - 1 + n;
    p.n_group1 = n;
    p.start2 = 0;
    p.end2 = -1;
    p.n_group2 = 0;
    int64_t offset = start - 1;
    double m = o.mass[s];
    double vscale = distribution == 1 ? std::sqrt(2.0 * k_B * T / m) * std::sqrt(0.3) : std::sqrt(2.0 * k_B * T / m);
    for (int64_t i = 1; i <= n; ++i) {
        orc_stream rng = orc_stream_make(seed, ORC_TAG_SAMPLE, (uint32_t)s, step, (uint32_t)(cell - 1), (uint32_t)(i - 1));
        update_particle_buffer_new_particle(pv, i + offset);
        Particle& q = pv.at(i + offset);
        q.w = Fnum;
        for (int c = 0; c < 3; ++c) q.x[c] = box[2 * c] + orc_stream_uniform(&rng) * (box[2 * c + 1] - box[2 * c]);
        pv.cell[i + offset - 1] = cell;
        if (distribution == 1)
            sample_bkw_one(&rng, q, vscale, v0);
        else
            sample_maxwellian_one(&rng, q, vscale, v0);
    }
}

}  // namespace

// ============================================================== C interface
extern "C" {

void* orc_create(int64_t n_cells, int32_t n_species)
{
    Orc* o = new Orc();
    o->n_cells = n_cells;
    o->n_species = n_species;
    o->pv.resize(n_species);
    o->indexer.assign(n_cells * n_species, empty_indexer());
    o->n_total.assign(n_species, 0);
    o->contiguous.assign(n_species, 1);
    o->mass.assign(n_species, 0.0);
    o->inter.resize((size_t)n_species * n_species);
    o->cf.assign((size_t)n_species * n_species * n_cells, CollisionFactors());
    return o;
}

void orc_destroy(void* h) { delete (Orc*)h; }

void orc_set_mass(void* h, const double* mass)
{
    Orc* o = (Orc*)h;
    for (int s = 0; s < o->n_species; ++s) o->mass[s] = mass[s];
}

// load_interaction_data (collision_utils.jl:159-202) from per-pair VHS data
// given as symmetric [i * ns + k] arrays.
void orc_load_interactions(void* h, const double* vhs_d, const double* vhs_o, const double* vhs_Tref)
{
    Orc* o = (Orc*)h;
    int ns = o->n_species;
    for (int i = 0; i < ns; ++i)
        for (int k = 0; k < ns; ++k) {
            if (i < k) continue;
            double mi = o->mass[i], mk = o->mass[k];
            double m_r = mi * mk / (mi + mk);
            double mu1 = mi / (mi + mk), mu2 = mk / (mi + mk);
            double d = vhs_d[i * ns + k], om = vhs_o[i * ns + k], Tr = vhs_Tref[i * ns + k];
            double muref = compute_mu_ref(0.5 * (mi + mk), om, Tr, d);
            double fac = compute_vhs_factor(Tr, d, om, m_r);
            o->inter[i + ns * k] = Interaction{m_r, mu1, mu2, d, om, Tr, muref, fac};
            o->inter[k + ns * i] = Interaction{m_r, mu2, mu1, d, om, Tr, muref, fac};
        }
}

void orc_get_interaction(void* h, int32_t s1, int32_t s2, double* rec)
{
    Orc* o = (Orc*)h;
    const Interaction& I = o->inter[s1 + o->n_species * s2];
    double r[8] = {I.m_r, I.mu1, I.mu2, I.vhs_d, I.vhs_o, I.vhs_Tref, I.vhs_muref, I.vhs_factor};
    std::memcpy(rec, r, sizeof r);
}

void orc_pv_create(void* h, int32_t s, int64_t np) { pv_init(((Orc*)h)->pv[s], np); }
void orc_set_cell_offset(void* h, int64_t offset) { ((Orc*)h)->cell_offset = offset; }
void orc_pv_resize(void* h, int32_t s, int64_t np) { pv_resize(((Orc*)h)->pv[s], np); }
int64_t orc_pv_length(void* h, int32_t s) { return ((Orc*)h)->pv[s].length(); }

void orc_pv_get(void* h, int32_t s, double* particles, int64_t* index, int64_t* cell, int64_t* buffer,
                int64_t* nbuffer)
{
    ParticleVector& pv = ((Orc*)h)->pv[s];
    int64_t n = pv.length();
    for (int64_t i = 0; i < n; ++i) {
        const Particle& q = pv.particles[i];
        double r[7] = {q.w, q.v[0], q.v[1], q.v[2], q.x[0], q.x[1], q.x[2]};
        std::memcpy(particles + 7 * i, r, sizeof r);
    }
    std::memcpy(index, pv.index.data(), n * sizeof(int64_t));
    std::memcpy(cell, pv.cell.data(), n * sizeof(int64_t));
    std::memcpy(buffer, pv.buffer.data(), n * sizeof(int64_t));
    *nbuffer = pv.nbuffer;
}

void orc_pv_set(void* h, int32_t s, int64_t n, const double* particles, const int64_t* index, const int64_t* cell,
                const int64_t* buffer, int64_t nbuffer)
{
    ParticleVector& pv = ((Orc*)h)->pv[s];
    pv.particles.resize(n);
    pv.index.assign(index, index + n);
    pv.cell.assign(cell, cell + n);
    pv.buffer.assign(buffer, buffer + n);
    pv.nbuffer = nbuffer;
    for (int64_t i = 0; i < n; ++i) {
        const double* r = particles + 7 * i;
        pv.particles[i] = Particle{r[0], {r[1], r[2], r[3]}, {r[4], r[5], r[6]}};
    }
}

void orc_pia_get(void* h, int64_t* indexer, int64_t* n_total, uint8_t* contiguous)
{
    Orc* o = (Orc*)h;
    for (size_t i = 0; i < o->indexer.size(); ++i) {
        const ParticleIndexer& p = o->indexer[i];
        int64_t r[7] = {p.n_local, p.start1, p.end1, p.n_group1, p.start2, p.end2, p.n_group2};
        std::memcpy(indexer + 7 * i, r, sizeof r);
    }
    for (int s = 0; s < o->n_species; ++s) {
        n_total[s] = o->n_total[s];
        contiguous[s] = o->contiguous[s];
    }
}

void orc_pia_set(void* h, const int64_t* indexer, const int64_t* n_total, const uint8_t* contiguous)
{
    Orc* o = (Orc*)h;
    for (size_t i = 0; i < o->indexer.size(); ++i) {
        const int64_t* r = indexer + 7 * i;
        o->indexer[i] = ParticleIndexer{r[0], r[1], r[2], r[3], r[4], r[5], r[6]};
    }
    for (int s = 0; s < o->n_species; ++s) {
        o->n_total[s] = n_total[s];
        o->contiguous[s] = contiguous[s];
    }
}

void orc_cf_get(void* h, int32_t s1, int32_t s2, double* smax, int64_t* counters)
{
    Orc* o = (Orc*)h;
    for (int64_t c = 1; c <= o->n_cells; ++c) {
        const CollisionFactors& f = o->cfa(s1, s2, c);
        smax[c - 1] = f.sigma_g_w_max;
        int64_t r[5] = {f.n1, f.n2, f.n_coll, f.n_coll_performed, f.n_eq_w_coll_performed};
        std::memcpy(counters + 5 * (c - 1), r, sizeof r);
    }
}

void orc_cf_set_smax(void* h, int32_t s1, int32_t s2, const double* smax)
{
    Orc* o = (Orc*)h;
    for (int64_t c = 1; c <= o->n_cells; ++c) o->cfa(s1, s2, c).sigma_g_w_max = smax[c - 1];
}

// estimate_sigma_g_w_max! (collision_utils.jl:464-504)
void orc_estimate_sigma_g_w_max(void* h, const double* T_list, const double* Fnum, int32_t fnum_per_species,
                                double mult)
{
    Orc* o = (Orc*)h;
    int ns = o->n_species;
    for (int k = 0; k < ns; ++k)
        for (int i = 0; i < ns; ++i) {
            double F = fnum_per_species ? std::max(Fnum[i], Fnum[k]) : Fnum[0];
            double v = estimate_sigma_g_w_max(o->inter[i + ns * k], o->mass[i], o->mass[k], T_list[i], T_list[k], F, mult);
            for (int64_t c = 1; c <= o->n_cells; ++c) o->cfa(i, k, c).sigma_g_w_max = v;
        }
}

double orc_estimate_sigma_g_w_max_single(void* h, int32_t s1, int32_t s2, double T1, double T2, double Fnum, double mult)
{
    Orc* o = (Orc*)h;
    return estimate_sigma_g_w_max(o->inter[s1 + o->n_species * s2], o->mass[s1], o->mass[s2], T1, T2, Fnum, mult);
}

// cell is 1-based, as in the reference.
void orc_ntc(void* h, int32_t s1, int32_t s2, int64_t cell, double dt, double V, uint64_t seed, uint64_t step,
             double dw_tol, int32_t equal_weight)
{
    Orc* o = (Orc*)h;
    if (s1 == s2)
        ntc_single(*o, s1, cell, dt, V, seed, step, dw_tol, equal_weight != 0);
    else
        ntc_two(*o, s1, s2, cell, dt, V, seed, step, dw_tol, equal_weight != 0);
}

// The per-cell loop of the drivers (e.g. simulations/1D/couette_benchmarking.jl:64-67).
// Cells are independent when no particle is split, so the equal-weight form
// may run cells on several threads.
void orc_ntc_cells(void* h, int32_t s1, int32_t s2, double dt, const double* V, uint64_t seed, uint64_t step,
                   double dw_tol, int32_t equal_weight, int32_t nthreads)
{
    Orc* o = (Orc*)h;
    int64_t nc = o->n_cells;
    if (equal_weight && nthreads > 1) {
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 16)
        for (int64_t c = 1; c <= nc; ++c) orc_ntc(h, s1, s2, c, dt, V ? V[c - 1] : 1.0, seed, step, dw_tol, 1);
    } else {
        for (int64_t c = 1; c <= nc; ++c) orc_ntc(h, s1, s2, c, dt, V ? V[c - 1] : 1.0, seed, step, dw_tol, equal_weight);
    }
}

// swpm! over every cell in order (the per-cell loop of
// test/test_1D_couette_varweight_swpm.jl:76-83 without the merging); V per
// cell, NULL for 1.0.  Cell is 1-based in orc_swpm.
void orc_swpm(void* h, int32_t s, int64_t cell, double G, double dt, double V, uint64_t seed, uint64_t step)
{
    swpm_cell(*(Orc*)h, s, cell, G, dt, V, seed, step);
}

void orc_swpm_cells(void* h, int32_t s, double G, double dt, const double* V, uint64_t seed, uint64_t step)
{
    Orc* o = (Orc*)h;
    for (int64_t c = 1; c <= o->n_cells; ++c) swpm_cell(*o, s, c, G, dt, V ? V[c - 1] : 1.0, seed, step);
}

// mode 0: compute_props!, 1: compute_props_with_total_moments!,
// 2: compute_props_sorted!, 3: compute_props_sorted!(..., grid) with number density
void orc_compute_props(void* h, int32_t mode, const int32_t* powers, int32_t n_mom, double Tref, const double* inv_V,
                       double* lpa, double* np, double* n, double* v, double* T, double* moments, int32_t nthreads)
{
    Orc* o = (Orc*)h;
    PropsOut out{lpa, np, n, v, T, moments};
    if (mode == 0)
        compute_props(*o, powers, 0, Tref, out, false, nthreads);
    else if (mode == 1)
        compute_props(*o, powers, n_mom, Tref, out, n_mom > 0, nthreads);
    else if (mode == 2)
        compute_props_sorted(*o, out, nullptr, nthreads);
    else
        compute_props_sorted(*o, out, inv_V, nthreads);
}

// avg_props! (physical_props.jl:281-299) over one flat array
void orc_avg_props(int64_t count, double* avg, const double* inst, double n_avg_timesteps)
{
    double inv = 1.0 / n_avg_timesteps;
    for (int64_t i = 0; i < count; ++i) avg[i] = std::fma(inst[i], inv, avg[i]);
}

// walls: [T_l, T_r, vl0, vl1, vl2, vr0, vr1, vr2, acc_l, acc_r]
// MaxwellWalls1D (boundary_conditions.jl:29-53) from the flat array
// {T_l, T_r, v_l[3], v_r[3], acc_l, acc_r}
static Walls make_walls(const Orc& o, const double* walls)
{
    Walls W;
    W.T[0] = walls[0];
    W.T[1] = walls[1];
    for (int c = 0; c < 3; ++c) {
        W.v[0][c] = walls[2 + c];
        W.v[1][c] = walls[5 + c];
    }
    W.acc[0] = walls[8];
    W.acc[1] = walls[9];
    W.vsq.resize(2 * o.n_species);
    for (int sp = 0; sp < o.n_species; ++sp) {
        W.vsq[0 + 2 * sp] = 2.0 * k_B * W.T[0] / o.mass[sp];
        W.vsq[1 + 2 * sp] = 2.0 * k_B * W.T[1] / o.mass[sp];
    }
    return W;
}

void orc_convect(void* h, int32_t s, double L, int64_t nx, double wall_offset, const double* walls, double dt,
                 uint64_t seed, uint64_t step, int32_t compute_cell, int32_t nthreads)
{
    Orc* o = (Orc*)h;
    Grid1D g = make_grid(L, nx, wall_offset);
    Walls W = make_walls(*o, walls);
    convect_particles(*o, s, g, W, dt, seed, step, compute_cell != 0, nthreads);
}

// convect_particles! with SurfProps: out[2][11] = the scaled surface sums of
// this call (surface_props.jl layout per element, see SQ_*)
void orc_convect_surf(void* h, int32_t s, double L, int64_t nx, double wall_offset, const double* walls, double dt,
                      uint64_t seed, uint64_t step, double* out)
{
    Orc* o = (Orc*)h;
    Grid1D g = make_grid(L, nx, wall_offset);
    Walls W = make_walls(*o, walls);
    Surf surf;
    convect_particles(*o, s, g, W, dt, seed, step, false, 1, &surf);
    for (int e = 0; e < 2; ++e)
        for (int k = 0; k < SQ_N; ++k) out[e * SQ_N + k] = surf.q[e][k];
}

// one incident (reflected = 0) or reflected update of element e of q[2][11]
void orc_surf_update(double* q, int32_t e, double w, const double* v, int32_t reflected)
{
    surf_update(q + e * SQ_N, e, w, v, reflected != 0);
}

void orc_surf_scale(double* q, double mass, double dt, const double* inv_areas)
{
    for (int e = 0; e < 2; ++e) surf_scale(q + e * SQ_N, mass, dt, inv_areas[e]);
}

void orc_grid(double L, int64_t nx, double wall_offset, double* out5)
{
    Grid1D g = make_grid(L, nx, wall_offset);
    out5[0] = g.dx;
    out5[1] = g.inv_dx;
    out5[2] = g.min_x;
    out5[3] = g.max_x;
    out5[4] = g.L;
}

// L <= 0: sort with stored cell ids
void orc_sort(void* h, int32_t s, double L, int64_t nx, double wall_offset)
{
    Orc* o = (Orc*)h;
    if (L > 0) {
        Grid1D g = make_grid(L, nx, wall_offset);
        sort_particles(*o, s, &g);
    } else {
        sort_particles(*o, s, nullptr);
    }
}

void orc_squash(void* h, int32_t s) { squash_pia(*(Orc*)h, s); }
void orc_restore_ordering(void* h, int32_t s) { restore_particle_ordering(((Orc*)h)->pv[s]); }
void orc_delete_particle_end(void* h, int32_t s, int64_t cell) { delete_particle_end(*(Orc*)h, cell, s); }
// map_cont_index (particles.jl:364-366): 0-based position within the cell's
// particles -> position in the index array (1-based)
int64_t orc_map_cont_index(void* h, int32_t s, int64_t cell, int64_t i) { return map_cont_index(((Orc*)h)->pi(cell, s), i); }
// update_particle_indexer_new_particle! (particles.jl:426-433)
void orc_indexer_new_particle(void* h, int32_t s, int64_t cell) { update_particle_indexer_new_particle(*(Orc*)h, cell, s); }
void orc_delete_particle_end_group(void* h, int32_t s, int64_t cell, int32_t group)
{
    if (group == 1)
        delete_particle_end_group1(*(Orc*)h, cell, s);
    else
        delete_particle_end_group2(*(Orc*)h, cell, s);
}

void* orc_octree_create(int32_t split, int32_t init_bounds, int32_t bounds_mode, int64_t max_Nbins, int64_t max_depth)
{
    return octree_new(split, init_bounds, bounds_mode, max_Nbins, max_depth);
}
void orc_octree_destroy(void* oc) { delete (Octree*)oc; }
void orc_octree_init(void* h, void* oc, int32_t s, int64_t cell)
{
    Orc* o = (Orc*)h;
    Octree* t = (Octree*)oc;
    t->Nbins = 0;
    resize_octree_buffers(*t, o->pi(cell, s).n_local);
    init_octree(*t, *o, s, cell);
}
void orc_octree_split(void* h, void* oc, int32_t s, int64_t bin_id) { split_bin(*(Octree*)oc, bin_id, ((Orc*)h)->pv[s]); }
void orc_octree_bin_props(void* h, void* oc, int32_t s, int64_t bin_id)
{
    compute_bin_props(*(Octree*)oc, bin_id, ((Orc*)h)->pv[s]);
}
void orc_octree_compute_v_mean(void* h, void* oc, int32_t s, int64_t bs, int64_t be)
{
    Octree* t = (Octree*)oc;
    for (int c = 0; c < 3; ++c) t->vel_middle[c] = 0.0;
    compute_v_mean(*t, bs, be, ((Orc*)h)->pv[s]);
}
void orc_octree_bounds_recompute(void* h, void* oc, int32_t s, int64_t bin_id, int64_t bs, int64_t be)
{
    bin_bounds_recompute(*(Octree*)oc, bin_id, bs, be, ((Orc*)h)->pv[s]);
}
// summary: [Nbins, n_particles, total_post_merge_np, vel_middle(3)]
void orc_octree_summary(void* oc, double* out6)
{
    Octree* t = (Octree*)oc;
    out6[0] = (double)t->Nbins;
    out6[1] = (double)t->n_particles;
    out6[2] = (double)t->total_post_merge_np;
    for (int c = 0; c < 3; ++c) out6[3 + c] = t->vel_middle[c];
}
void orc_octree_pis(void* oc, int64_t n, int64_t* out)
{
    Octree* t = (Octree*)oc;
    for (int64_t i = 0; i < n; ++i) out[i] = t->pis[i];
}
// per bin: [np, w, depth, can_be_refined, bin_start, bin_end, vmin(3), vmax(3), v_mean(3), x_mean(3)] = 18
void orc_octree_bins(void* oc, int64_t nbins, double* out)
{
    Octree* t = (Octree*)oc;
    for (int64_t b = 0; b < nbins; ++b) {
        const OctreeCell& c = t->bins[b];
        const OctreeFullCell& f = t->full_bins[b];
        double* r = out + 18 * b;
        r[0] = (double)c.np;
        r[1] = c.w;
        r[2] = (double)c.depth;
        r[3] = c.can_be_refined ? 1.0 : 0.0;
        r[4] = (double)t->bin_start[b];
        r[5] = (double)t->bin_end[b];
        for (int k = 0; k < 3; ++k) {
            r[6 + k] = c.vmin[k];
            r[9 + k] = c.vmax[k];
            r[12 + k] = f.v_mean[k];
            r[15 + k] = f.x_mean[k];
        }
    }
}

// merge_octree_N2_based!; L <= 0 selects the variant without a grid
void orc_merge_octree(void* h, void* oc, int32_t s, int64_t cell, int64_t target, double L, int64_t nx,
                      double wall_offset, uint64_t seed, uint64_t step)
{
    Orc* o = (Orc*)h;
    if (L > 0) {
        Grid1D g = make_grid(L, nx, wall_offset);
        merge_octree_N2_based(*(Octree*)oc, *o, s, cell, target, &g, seed, step);
    } else {
        merge_octree_N2_based(*(Octree*)oc, *o, s, cell, target, nullptr, seed, step);
    }
}

// check_pia_is_correct (particles.jl:863-907): returns 1 if correct; *bad = cell or 0
int32_t orc_check_pia(void* h, int32_t s, int64_t* bad)
{
    Orc* o = (Orc*)h;
    int64_t n_tot = 0;
    for (int64_t i = 1; i <= o->n_cells; ++i) {
        const ParticleIndexer& p = o->pi(i, s);
        *bad = i;
        if (p.n_local != p.n_group1 + p.n_group2) return 0;
        n_tot += p.n_local;
        if (p.n_group1 > 0) {
            if (p.n_group1 != p.end1 - p.start1 + 1) return 0;
        } else if (p.start1 != 0 || p.end1 != -1) {
            return 0;
        }
        if (p.n_group2 > 0) {
            if (p.n_group2 != p.end2 - p.start2 + 1) return 0;
        } else if (p.start2 != 0 || p.end2 != -1) {
            return 0;
        }
    }
    *bad = 0;
    return n_tot == o->n_total[s] ? 1 : 0;
}

// check_unique_index (particles.jl:942-986): returns the reference's second value
int64_t orc_check_unique_index(void* h, int32_t s)
{
    Orc* o = (Orc*)h;
    ParticleVector& pv = o->pv[s];
    std::vector<int64_t> counts(pv.index.size() + 1, 0);
    int64_t retcode = 1;
    for (int64_t c = 1; c <= o->n_cells; ++c) {
        const ParticleIndexer& p = o->pi(c, s);
        for (int64_t i = p.start1; i <= p.end1; ++i) counts[pv.index[i - 1]] += 1;
        for (int64_t i = p.start2; i <= p.end2; ++i) counts[pv.index[i - 1]] += 1;
    }
    int64_t n_index = *std::max_element(counts.begin(), counts.end());
    for (int64_t i = 0; i < pv.nbuffer; ++i)
        if (counts[pv.buffer[i]] > 0) {
            retcode = -1;
            break;
        }
    if (n_index > 1) return n_index * retcode;
    if (retcode == -1) return -1;
    return 0;
}

// check_unique_buffer (particles.jl:1009-1025): 0 if correct, else position
int64_t orc_check_unique_buffer(void* h, int32_t s)
{
    ParticleVector& pv = ((Orc*)h)->pv[s];
    std::vector<uint8_t> seen(pv.index.size() + 1, 0);
    for (int64_t i = 1; i <= pv.nbuffer; ++i) {
        int64_t pid = pv.buffer[i - 1];
        if (seen[pid]) return i;
        seen[pid] = 1;
    }
    return 0;
}

// sample_particles_equal_weight! for one cell; distribution 0 = Maxwellian, 1 = BKW
void orc_sample_particles_equal_weight(void* h, int32_t s, int64_t cell, int64_t n, double T, double Fnum,
                                       const double* box6, uint64_t seed, uint64_t step, int32_t distribution,
                                       const double* v0)
{
    sample_particles_equal_weight(*(Orc*)h, s, cell, n, T, Fnum, box6, seed, step, distribution, v0);
}

// sample_particles_equal_weight!(rng, grid, ..., ndens::Float64, T, Fnum),
// grid_uniform1D.jl:198-219; the fractional extra particle uses its own stream.
void orc_sample_grid_ndens(void* h, int32_t s, double L, int64_t nx, double wall_offset, double ndens, double T,
                           double Fnum, uint64_t seed, uint64_t step, const double* v0_in)
{
    Orc* o = (Orc*)h;
    Grid1D g = make_grid(L, nx, wall_offset);
    // the keywords vx0, vy0, vz0 of grid_uniform1D.jl:215-219
    double v0[3] = {0, 0, 0};
    if (v0_in)
        for (int k = 0; k < 3; ++k) v0[k] = v0_in[k];
    for (int64_t cell = 1; cell <= nx; ++cell) {
        double xlo = (double)(cell - 1) * g.dx, xhi = (double)cell * g.dx;
        double n_in_cell = ndens * g.dx;
        double ppc = n_in_cell / Fnum;
        int64_t ppc_int = (int64_t)std::floor(ppc);
        double remainder = ppc - (double)ppc_int;
        orc_stream r = orc_stream_make(seed, ORC_TAG_SAMPLE_CELL, (uint32_t)s, step, (uint32_t)(cell - 1), 0);
        if (orc_stream_uniform(&r) < remainder) ppc_int += 1;
        double box[6] = {xlo, xhi, 0.0, 1.0, 0.0, 1.0};
        sample_particles_equal_weight(*o, s, cell, ppc_int, T, Fnum, box, seed, step, 0, v0);
    }
}

// uniform draws of one stream (for RNG parity tests)
void orc_stream_draws(uint64_t seed, uint32_t tag, uint32_t sub, uint64_t step, uint32_t a, uint32_t b, int64_t n,
                      double* out)
{
    orc_stream s = orc_stream_make(seed, tag, sub, step, a, b);
    for (int64_t i = 0; i < n; ++i) out[i] = orc_stream_uniform(&s);
}

void orc_philox(const uint32_t* ctr, const uint32_t* key, uint32_t* out) { orc_philox4x32_10(ctr, key, out); }

// Unit hooks mirroring the reference's unit tests
// (test/test_collision_utils.jl:19-40): compute_com!, compute_g!, scatter_vhs!.
// p1, p2: 7 doubles each, updated in place.  out4 = [vcom(3), g] before scattering.
void orc_com_g_scatter(void* h, int32_t s1, int32_t s2, double* p1, double* p2, uint64_t seed, int32_t do_scatter,
                       double* out4)
{
    Orc* o = (Orc*)h;
    const Interaction& I = o->inter[s1 + o->n_species * s2];
    Particle a{p1[0], {p1[1], p1[2], p1[3]}, {p1[4], p1[5], p1[6]}};
    Particle b{p2[0], {p2[1], p2[2], p2[3]}, {p2[4], p2[5], p2[6]}};
    CollisionData cd;
    compute_com(cd, I, a, b);
    compute_g(cd, a, b);
    for (int c = 0; c < 3; ++c) out4[c] = cd.v_com[c];
    out4[3] = cd.g;
    if (do_scatter) {
        orc_stream rng = orc_stream_make(seed, ORC_TAG_CAND, 0, 0, 0, 0);
        scatter_vhs(&rng, cd, I, a, b);
    }
    double ra[7] = {a.w, a.v[0], a.v[1], a.v[2], a.x[0], a.x[1], a.x[2]};
    double rb[7] = {b.w, b.v[0], b.v[1], b.v[2], b.x[0], b.x[1], b.x[2]};
    std::memcpy(p1, ra, sizeof ra);
    std::memcpy(p2, rb, sizeof rb);
}

// collide_2particles_vhs! on ParticleVector positions pos_i (species s1) and
// pos_k (species s2) of `cell` (test/test_collision_vhs.jl:57-59 and siblings).
// Uses the candidate-0 stream of step 0; the cell's sigma_g_w_max is the
// CollisionFactors value stored in the state.
void orc_collide_vhs(void* h, int32_t s1, int32_t s2, int64_t cell, int64_t pos_i, int64_t pos_k, double dw_tol,
                     uint64_t seed, int32_t equal_weight)
{
    Orc* o = (Orc*)h;
    CollisionFactors& cf = o->cfa(s1, s2, cell);
    const Interaction& I = o->inter[s1 + o->n_species * s2];
    orc_stream rng = orc_stream_make(seed, ORC_TAG_CAND, pair_code(*o, s1, s2), 0, (uint32_t)(cell - 1), 0);
    int64_t phys_i = o->pv[s1].index[pos_i - 1] - 1;
    int64_t phys_k = o->pv[s2].index[pos_k - 1] - 1;
    CollisionData cd;
    compute_g(cd, o->pv[s1].particles[phys_i], o->pv[s2].particles[phys_k]);
    if (equal_weight)
        collide_2particles_vhs_equal_weight(&rng, cd, cf, I, o->pv[s1].particles[phys_i], o->pv[s2].particles[phys_k]);
    else
        collide_2particles_vhs(&rng, cd, cf, I, *o, phys_i, phys_k, s1, s2, cell, dw_tol);
}

int32_t orc_compute_octant(const double* v, const double* mid) { return compute_octant(v, mid); }

double orc_tgamma(double x) { return std::tgamma(x); }

}  // extern "C"
