// Moment reductions: compute_props! (physical_props.jl:104-154),
// compute_props_with_total_moments! (:168-245), compute_props_sorted! (:317-354,
// number-density variant :393-433), avg_props! (:281-299), clear_props! (:256-262).
//
// One warp per (cell, species): pass 1 sums w and w*v over the cell's logical
// list, pass 2 sums w*|v - u|^2 (and w*|v - u|^m).  Each lane accumulates a
// strided subset; a butterfly reduction combines the lanes.  Outputs use
// Merzbild's column-major PhysProps layouts.
// Algorithmic bytes per particle: 32 read (w, vx, vy, vz) per pass.
#include "cell_ops.cuh"
#include "mz_host.h"

#include <algorithm>

using namespace mz;

namespace {

struct PropsView {
    double *np, *n, *v, *T, *moments;
    int32_t n_moments;
    int32_t powers[16];
    double Tref;
    int32_t ndens;
};

__global__ void __launch_bounds__(256) k_props(DomainView d, PropsView P, int mode)
{
    const int lane = threadIdx.x & 31;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const int nc = d.n_cells;
    const int total = nc * d.n_species;
    const bool with_mom = (mode == MZ_PROPS_MOMENTS) && P.n_moments > 0;
    for (int wi = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; wi < total; wi += nwarps) {
        const int s = wi / nc, c = wi - s * nc;
        const SpeciesView& S = d.sp[s];
        const Indexer p = S.ind[c];
        const int32_t nl = (mode == MZ_PROPS_SORTED) ? p.n1 : p.n1 + p.n2;
        double mom[16];
        double n, ux, uy, uz, T;
        if (!with_mom) {
            const CellMoments r = props_cell(S.A, p, nl, S.mass);
            n = r.n;
            ux = r.ux;
            uy = r.uy;
            uz = r.uz;
            T = r.T;
        } else {
            n = 0.0;
            double sx = 0.0, sy = 0.0, sz = 0.0;
            for (int j = lane; j < nl; j += 32) {
                const PV r = S.A.wv[map_slot(p, j)];
                n += r.w;
                sx += r.vx * r.w;
                sy += r.vy * r.w;
                sz += r.vz * r.w;
            }
            n = warp_sum(n);
            sx = warp_sum(sx);
            sy = warp_sum(sy);
            sz = warp_sum(sz);
            ux = uy = uz = T = 0.0;
            for (int m = 0; m < 16; ++m) mom[m] = 0.0;
            if (n > 0.0) {
                ux = sx / n;
                uy = sy / n;
                uz = sz / n;
                double E = 0.0;
                for (int j = lane; j < nl; j += 32) {
                    const PV r = S.A.wv[map_slot(p, j)];
                    const double w = r.w;
                    const double dx = r.vx - ux, dy = r.vy - uy, dz = r.vz - uz;
                    const double nv = sqrt((dx * dx + dy * dy) + dz * dz);
                    E = fma(w, nv * nv, E);
                    for (int m = 0; m < P.n_moments; ++m) mom[m] = fma(w, pow(nv, (double)P.powers[m]), mom[m]);
                }
                E = warp_sum(E);
                for (int m = 0; m < P.n_moments; ++m) mom[m] = warp_sum(mom[m]);
                E *= 0.5 * S.mass / (n * K_B);
                T = (2.0 / 3.0) * E;
            }
        }
        if (lane == 0) {
            const int64_t ix = (int64_t)c + (int64_t)nc * s;
            P.np[ix] = (double)nl;
            P.n[ix] = (P.ndens && mode == MZ_PROPS_SORTED) ? n * (1.0 / d.cell_V[c]) : n;
            P.v[3 * ix + 0] = ux;
            P.v[3 * ix + 1] = uy;
            P.v[3 * ix + 2] = uz;
            P.T[ix] = T;
            if (with_mom) {
                const double mass = S.mass;
                const double factor = 4.0 * 3.141592653589793 * pow(mass / (TWOPI * K_B * P.Tref), 1.5) * 0.5;
                const double vref = pow(mass / (2.0 * K_B * P.Tref), 0.5);
                for (int m = 0; m < P.n_moments; ++m) {
                    const double mm = (double)P.powers[m];
                    const double scaling = factor * pow(vref, -(3.0 + mm)) * tgamma((3.0 + mm) / 2.0);
                    P.moments[m + (int64_t)P.n_moments * ix] = mom[m] / (scaling * n);
                }
            }
        }
    }
}

__global__ void k_avg(double* avg, const double* inst, int64_t n, double inv)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        avg[i] = fma(inst[i], inv, avg[i]);
}

}  // namespace

static PropsView make_props_view(mz_props* p)
{
    PropsView v;
    v.np = p->np;
    v.n = p->n;
    v.v = p->v;
    v.T = p->T;
    v.moments = p->moments;
    v.n_moments = p->n_moments;
    for (int i = 0; i < 16; ++i) v.powers[i] = p->powers[i];
    v.Tref = p->Tref;
    v.ndens = p->ndens;
    return v;
}

void launch_props(mz_domain* d, mz_props* p, int32_t mode)
{
    mz_ctx* c = d->ctx;
    DomainView v = make_view(d);
    const int64_t total = d->n_cells * d->ns;
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(div_up(total * 32, 256), (int64_t)c->num_sms * 16));
    MZ_LAUNCH(c, "props", k_props, blocks, 256, 0, v, make_props_view(p), (int)mode);
    for (int s = 0; s < d->ns; ++s)
        if (mode != MZ_PROPS_SORTED) p->lpa[s] = (double)d->sp[s].capacity;
}

void launch_avg(mz_ctx* c, double* avg, const double* inst, int64_t n, double inv)
{
    if (n <= 0 || !avg || !inst) return;
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(div_up(n, 256), (int64_t)c->num_sms * 8));
    MZ_LAUNCH(c, "avg_props", k_avg, blocks, 256, 0, avg, inst, n, inv);
}
