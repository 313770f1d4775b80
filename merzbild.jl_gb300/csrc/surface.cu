// Surface properties of the walls of a 1-D grid: SurfProps(pia, grid),
// clear_props!, avg_props! and surface_props_scale! (surface_props.jl:22-67,
// :149-253), convect_particles! with surface sampling (convection_1D.jl:
// 72-112, 176-206), and the fused step's per-step sampling.
//
// Wall hits add their incident and reflected contributions to per-thread sums
// that each block adds to the device sums atomically (cell_ops.cuh), so the
// order of the additions -- unlike the reference's particle order -- varies
// between runs: the sums agree with the sequential ones to round-off.
#include "cell_ops.cuh"
#include "mz_host.h"

#include <algorithm>

using namespace mz;

namespace {

// surface_props_scale!: every quantity but np times mass / dt / area (area 1)
__global__ void k_surf_scale(double* acc, int s_begin, int s_end, const double* factor)
{
    const int t = threadIdx.x;
    for (int s = s_begin; s < s_end; ++s)
        if (t < 2 * SURF_Q && (t % SURF_Q) != 0) acc[(size_t)s * 2 * SURF_Q + t] *= factor[s];
}

__global__ void k_surf_avg(double* avg, const double* inst, int n, double inv)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        avg[i] = fma(inst[i], inv, avg[i]);
}

}  // namespace

// scale species [s_begin, s_end) of a surface set by mass / dt (device side)
void launch_surf_scale(mz_domain* d, mz_surf_props* sp, int s_begin, int s_end, double dt)
{
    double f[MZ_MAX_SPECIES] = {0, 0, 0, 0};
    for (int s = 0; s < d->ns; ++s) f[s] = d->mass[s] / dt;
    double* df = reinterpret_cast<double*>(d->d_scalar + 4);  // 4 doubles of scratch
    static_assert(MZ_MAX_SPECIES <= 4, "scratch");
    MZ_CK(cudaMemcpyAsync(df, f, sizeof f, cudaMemcpyHostToDevice, d->ctx->stream));
    MZ_LAUNCH(d->ctx, "surf_scale", k_surf_scale, 1, 32, 0, sp->acc, s_begin, s_end, df);
}

extern "C" {

int mz_surf_props_create(mz_domain* d, mz_surf_props** out)
{
    mz_surf_props* p = nullptr;
    API_TRY
    MZ_REQUIRE(d && out, "mz_surf_props_create: NULL argument");
    MZ_CK(cudaSetDevice(d->ctx->device));
    p = new mz_surf_props_s();
    p->dom = d;
    MZ_CK(cudaMalloc(&p->acc, (size_t)d->ns * 2 * SURF_Q * sizeof(double)));
    MZ_CK(cudaMemsetAsync(p->acc, 0, (size_t)d->ns * 2 * SURF_Q * sizeof(double), d->ctx->stream));
    d->surf.push_back(p);
    *out = p;
    p = nullptr;
    API_CATCH(d->ctx)
}

int mz_surf_props_destroy(mz_surf_props* p)
{
    if (!p) return MZ_OK;
    mz_domain* d = p->dom;
    cudaSetDevice(d->ctx->device);
    cudaStreamSynchronize(d->ctx->stream);
    cudaFree(p->acc);
    d->surf.erase(std::remove(d->surf.begin(), d->surf.end(), p), d->surf.end());
    if (d->step_surf == p) d->step_surf = nullptr;
    if (d->step_surf_avg == p) d->step_surf_avg = nullptr;
    delete p;
    return MZ_OK;
}

int mz_surf_props_clear(mz_surf_props* p)
{
    API_TRY
    MZ_REQUIRE(p, "mz_surf_props_clear: NULL");
    mz_domain* d = p->dom;
    MZ_CK(cudaMemsetAsync(p->acc, 0, (size_t)d->ns * 2 * SURF_Q * sizeof(double), d->ctx->stream));
    API_CATCH(p->dom->ctx)
}

int mz_surf_avg_props(mz_surf_props* avg, const mz_surf_props* inst, double n_avg_timesteps)
{
    API_TRY
    MZ_REQUIRE(avg && inst && avg->dom == inst->dom && n_avg_timesteps > 0, "mz_surf_avg_props: bad argument");
    mz_domain* d = avg->dom;
    const int n = d->ns * 2 * SURF_Q;
    MZ_LAUNCH(d->ctx, "surf_avg", k_surf_avg, 1, 256, 0, avg->acc, inst->acc, n, 1.0 / n_avg_timesteps);
    API_CATCH(avg->dom->ctx)
}

int mz_surf_props_download(mz_surf_props* p, double* np, double* flux_incident, double* flux_reflected, double* force,
                           double* normal_pressure, double* shear_pressure, double* kinetic_energy_flux)
{
    API_TRY
    MZ_REQUIRE(p, "mz_surf_props_download: NULL");
    mz_domain* d = p->dom;
    const int ns = d->ns;
    std::vector<double> a((size_t)ns * 2 * SURF_Q);
    MZ_CK(cudaMemcpyAsync(a.data(), p->acc, a.size() * sizeof(double), cudaMemcpyDeviceToHost, d->ctx->stream));
    MZ_CK(cudaStreamSynchronize(d->ctx->stream));
    for (int s = 0; s < ns; ++s)
        for (int e = 0; e < 2; ++e) {
            const double* q = a.data() + ((size_t)s * 2 + e) * SURF_Q;
            const int ix = e + 2 * s;  // (n_elements, n_species), column-major
            if (np) np[ix] = q[0];
            if (flux_incident) flux_incident[ix] = q[1];
            if (flux_reflected) flux_reflected[ix] = q[2];
            for (int k = 0; k < 3; ++k) {
                if (force) force[k + 3 * ix] = q[3 + k];
                if (shear_pressure) shear_pressure[k + 3 * ix] = q[7 + k];
            }
            if (normal_pressure) normal_pressure[ix] = q[6];
            if (kinetic_energy_flux) kinetic_energy_flux[ix] = q[10];
        }
    API_CATCH(p->dom->ctx)
}

int mz_convect_1d_surf(mz_domain* d, int32_t s, const mz_grid1d* g, const mz_walls1d* w, double dt, uint64_t step,
                       int32_t flags, mz_surf_props* surf)
{
    API_TRY
    MZ_REQUIRE(d && g && w && surf && surf->dom == d, "mz_convect_1d_surf: bad argument");
    MZ_REQUIRE(s >= 0 && s < d->ns, "mz_convect_1d_surf: bad species");
    MZ_REQUIRE(g->n_cells == d->n_cells || (!(flags & MZ_CONVECT_COMPUTE_CELL) && g->n_cells > d->n_cells),
               "mz_convect_1d_surf: grid and domain cell counts differ");
    MZ_CK(cudaSetDevice(d->ctx->device));
    double* acc = surf->acc + (size_t)s * 2 * SURF_Q;
    MZ_CK(cudaMemsetAsync(acc, 0, 2 * SURF_Q * sizeof(double), d->ctx->stream));
    launch_convect(d, s, g, w, dt, step, flags, acc);
    launch_surf_scale(d, surf, s, s + 1, dt);
    check_status(d);
    API_CATCH(d->ctx)
}

int mz_step_set_surface(mz_domain* d, mz_surf_props* inst, mz_surf_props* avg)
{
    API_TRY
    MZ_REQUIRE(d, "mz_step_set_surface: NULL domain");
    MZ_REQUIRE((!inst || inst->dom == d) && (!avg || avg->dom == d), "mz_step_set_surface: sets of another domain");
    MZ_REQUIRE(!avg || inst, "mz_step_set_surface: averaging needs the instantaneous set");
    d->step_surf = inst;
    d->step_surf_avg = avg;
    API_CATCH(d->ctx)
}

}  // extern "C"
