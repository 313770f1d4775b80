// Initial-condition samplers: sample_particles_equal_weight! for a cell
// (distributions_and_sampling.jl:477-509) with sample_maxwellian! (:432-443)
// or sample_bkw! (:195-213), and the grid / number-density form
// (grid_uniform1D.jl:198-219).  Extensions used by the benchmark
// configurations (not in the reference): per-axis temperatures (a
// bi-Maxwellian) and log-uniform weights.
//
// Every particle draws from its own stream keyed on (cell, particle #), one
// thread per particle:
// 3 position draws, then the velocity draws, then one weight draw if the
// weights are log-uniform.  log(1 - U) replaces log(U) so U == 0 cannot give
// an infinite speed.
#include "mz_host.h"

#include <algorithm>

using namespace mz;

namespace {

struct SampleArgs {
    const int32_t* counts;
    const int32_t* base;
    const double* T3;     // n_cells x 3 or nullptr
    double T3_all[3];
    const double* Fnum;   // n_cells
    double span;
    const double* box6;   // n_cells x 6 or nullptr
    int grid_box;         // 1: box from the grid (dx)
    double dx;
    int dist;             // 0 Maxwellian, 1 BKW
    uint32_t step;
    const double* v0;     // n_cells x 3 velocity offsets (vx0, vy0, vz0) or nullptr
    double v0_all[3];     // the offset of every cell when v0 is nullptr
};

// indexers of the sampled cells (lists appended at base[c])
__global__ void k_sample_cells(DomainView d, int s, SampleArgs a)
{
    const SpeciesView& S = d.sp[s];
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < d.n_cells; c += gridDim.x * blockDim.x) {
        const int32_t n = a.counts[c];
        if (n <= 0) continue;
        const Indexer old = S.ind[c];
        if (old.n1 + old.n2 != 0) set_status(d, ST_CAPACITY);
        S.ind[c] = Indexer{a.base[c], n, 0, 0};
    }
}

// One thread per new particle (a cell of 10^5 particles spreads over the
// whole GPU); the particle's cell is found by bisection of the cell bases, and
// its stream is keyed on (cell, particle # in the cell) as before.
__global__ void __launch_bounds__(256) k_sample(DomainView d, int s, SampleArgs a, int64_t hw, int64_t total)
{
    const SpeciesView& S = d.sp[s];
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < total; g += (int64_t)gridDim.x * blockDim.x) {
        const int64_t x = hw + g;
        // last cell c with base[c] <= x (cells without particles share their successor's base)
        int lo = 0, hi = d.n_cells - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if ((int64_t)a.base[mid] <= x) lo = mid;
            else hi = mid - 1;
        }
        const int c = lo;
        const int32_t j = (int32_t)(x - a.base[c]);
        double lo3[3], hi3[3];
        if (a.grid_box) {
            lo3[0] = (double)c * a.dx;
            hi3[0] = (double)(c + 1) * a.dx;
            lo3[1] = 0.0;
            hi3[1] = 1.0;
            lo3[2] = 0.0;
            hi3[2] = 1.0;
        } else if (a.box6) {
            for (int k = 0; k < 3; ++k) {
                lo3[k] = a.box6[6 * (int64_t)c + 2 * k];
                hi3[k] = a.box6[6 * (int64_t)c + 2 * k + 1];
            }
        } else {
            for (int k = 0; k < 3; ++k) {
                lo3[k] = 0.0;
                hi3[k] = 1.0;
            }
        }
        double T[3];
        for (int k = 0; k < 3; ++k) T[k] = a.T3 ? a.T3[3 * (int64_t)c + k] : a.T3_all[k];
        const double Fn = a.Fnum[c];
        Stream st;
        st.init(cell_seed(d, c), TAG_SAMPLE, (uint32_t)s, cell_step(d, c, a.step), cell_rid(d, c), (uint32_t)j);
        const int64_t q = x;
        double xx[3];
        for (int k = 0; k < 3; ++k) xx[k] = lo3[k] + st.uniform() * (hi3[k] - lo3[k]);
        double vx, vy, vz;
        if (a.dist == 1) {
            const double vs = sqrt(2.0 * K_B * T[0] / S.mass) * sqrt(0.3);
            double z[6];
            for (int k = 0; k < 3; ++k) {
                const double r = sqrt(-2.0 * log(1.0 - st.uniform()));
                const double ang = TWOPI * st.uniform();
                z[2 * k] = r * cos(ang);
                z[2 * k + 1] = r * sin(ang);
            }
            const double vabs = sqrt(z[0] * z[0] + z[1] * z[1] + z[2] * z[2] + z[3] * z[3] + z[4] * z[4]);
            const double th = st.uniform() * 3.141592653589793;
            const double ph = st.uniform() * TWOPI;
            const double sth = sin(th);
            vx = vs * (vabs * sth * cos(ph));
            vy = vs * (vabs * sth * sin(ph));
            vz = vs * (vabs * cos(th));
        } else {
            const double vn = sqrt(-log(1.0 - st.uniform()));
            const double vr = sqrt(-log(1.0 - st.uniform()));
            const double t1 = TWOPI * st.uniform();
            const double t2 = TWOPI * st.uniform();
            vx = sqrt(2.0 * K_B * T[0] / S.mass) * (vn * cos(t1));
            vy = sqrt(2.0 * K_B * T[1] / S.mass) * (vr * cos(t2));
            vz = sqrt(2.0 * K_B * T[2] / S.mass) * (vr * sin(t2));
        }
        // the velocity offset of the keywords vx0, vy0, vz0
        // (distributions_and_sampling.jl:498-508)
        if (a.v0) {
            vx += a.v0[3 * (int64_t)c];
            vy += a.v0[3 * (int64_t)c + 1];
            vz += a.v0[3 * (int64_t)c + 2];
        } else {
            vx += a.v0_all[0];
            vy += a.v0_all[1];
            vz += a.v0_all[2];
        }
        double w = Fn;
        if (a.span > 0.0) w = Fn * pow(10.0, a.span * (2.0 * st.uniform() - 1.0));
        S.A.wv[q] = PV{w, vx, vy, vz};
        S.A.pos[q] = PX{xx[0], xx[1], xx[2], 0.0};
        S.cell[q] = c;
        S.key[q] = c;
    }
}

// per-cell particle count of the number-density sampler (grid_uniform1D.jl:198-211)
__global__ void k_grid_counts(DomainView d, int s, double ndens, double V, double Fnum, uint32_t step, int32_t* counts)
{
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < d.n_cells; c += gridDim.x * blockDim.x) {
        const double n_in_cell = ndens * V;
        const double ppc = n_in_cell / Fnum;
        double fl = floor(ppc);
        int32_t ppc_int = (int32_t)fl;
        const double rem = ppc - fl;
        Stream st;
        st.init(cell_seed(d, c), TAG_SAMPLE_CELL, (uint32_t)s, cell_step(d, c, step), cell_rid(d, c), 0);
        if (st.uniform() < rem) ppc_int += 1;
        counts[c] = ppc_int;
    }
}

}  // namespace

static void run_sample(mz_domain* d, int s, SampleArgs a, int32_t* counts_dev)
{
    mz_ctx* c = d->ctx;
    SpeciesHost& S = d->sp[s];
    // base[c] = hw + exclusive prefix of counts
    launch_scan_cells(d, counts_dev, S.ind, S.fill, d->d_scalar, false, S.work, S.hw);
    MZ_CK(cudaMemcpyAsync(d->h_scalar, d->d_scalar, sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
    MZ_CK(cudaStreamSynchronize(c->stream));
    const int64_t total = d->h_scalar[0];
    if (S.hw + total > S.capacity) reserve_species(d, s, S.hw + total);
    a.counts = counts_dev;
    a.base = S.work;
    DomainView v = make_view(d);
    const int cb = (int)std::max<int64_t>(1, std::min<int64_t>(div_up(d->n_cells, 256), (int64_t)c->num_sms * 8));
    MZ_LAUNCH(c, "sample_cells", k_sample_cells, cb, 256, 0, v, s, a);
    if (total > 0) {
        const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(div_up(total, 256), (int64_t)c->num_sms * 16));
        MZ_LAUNCH(c, "sample", k_sample, blocks, 256, 0, v, s, a, S.hw, total);
    }
    S.hw += total;
    S.n_total += total;
}

void launch_sample_cells(mz_domain* d, int s, const int64_t* counts_host, const int32_t* /*counts_dev*/,
                         const double* T3, const double* T3_all, const double* Fnum, double span, const double* box6,
                         int32_t distribution, uint64_t step, const double* v0, const double* v0_all)
{
    mz_ctx* c = d->ctx;
    const int64_t nc = d->n_cells;
    std::vector<int32_t> cnt(nc);
    for (int64_t i = 0; i < nc; ++i) {
        MZ_REQUIRE(counts_host[i] >= 0 && counts_host[i] < (1ll << 31), "mz_sample_cells: bad count");
        cnt[i] = (int32_t)counts_host[i];
    }
    // device staging: counts -> species fill array (free outside the sort)
    SpeciesHost& S = d->sp[s];
    MZ_CK(cudaMemcpyAsync(S.fill, cnt.data(), nc * sizeof(int32_t), cudaMemcpyHostToDevice, c->stream));
    double *dT3 = nullptr, *dF = nullptr, *dB = nullptr, *dV0 = nullptr;
    MZ_CK(cudaMalloc(&dF, nc * sizeof(double)));
    MZ_CK(cudaMemcpyAsync(dF, Fnum, nc * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    if (T3) {
        MZ_CK(cudaMalloc(&dT3, 3 * nc * sizeof(double)));
        MZ_CK(cudaMemcpyAsync(dT3, T3, 3 * nc * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    }
    if (box6) {
        MZ_CK(cudaMalloc(&dB, 6 * nc * sizeof(double)));
        MZ_CK(cudaMemcpyAsync(dB, box6, 6 * nc * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    }
    if (v0) {
        MZ_CK(cudaMalloc(&dV0, 3 * nc * sizeof(double)));
        MZ_CK(cudaMemcpyAsync(dV0, v0, 3 * nc * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    }
    SampleArgs a{};
    a.v0 = dV0;
    for (int k = 0; k < 3; ++k) a.v0_all[k] = v0_all ? v0_all[k] : 0.0;
    a.T3 = dT3;
    for (int k = 0; k < 3; ++k) a.T3_all[k] = T3_all ? T3_all[k] : 0.0;
    a.Fnum = dF;
    a.span = span;
    a.box6 = dB;
    a.grid_box = 0;
    a.dist = distribution;
    a.step = (uint32_t)step;
    try {
        run_sample(d, s, a, S.fill);
        MZ_CK(cudaStreamSynchronize(c->stream));
    } catch (...) {
        cudaFree(dF);
        cudaFree(dT3);
        cudaFree(dB);
        cudaFree(dV0);
        throw;
    }
    cudaFree(dF);
    cudaFree(dT3);
    cudaFree(dB);
    cudaFree(dV0);
}

void launch_sample_grid(mz_domain* d, int s, const mz_grid1d* g, double ndens, double T, double Fnum, uint64_t step,
                        const double* v0_all)
{
    mz_ctx* c = d->ctx;
    const int64_t nc = d->n_cells;
    SpeciesHost& S = d->sp[s];
    DomainView v = make_view(d);
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(div_up(nc, 256), (int64_t)c->num_sms * 8));
    MZ_LAUNCH(c, "sample_counts", k_grid_counts, blocks, 256, 0, v, s, ndens, g->dx, Fnum, (uint32_t)step, S.fill);
    double* dF = nullptr;
    MZ_CK(cudaMalloc(&dF, nc * sizeof(double)));
    std::vector<double> F(nc, Fnum);
    MZ_CK(cudaMemcpyAsync(dF, F.data(), nc * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    SampleArgs a{};
    a.T3 = nullptr;
    a.T3_all[0] = a.T3_all[1] = a.T3_all[2] = T;
    a.Fnum = dF;
    a.span = 0.0;
    a.box6 = nullptr;
    a.grid_box = 1;
    a.dx = g->dx;
    a.dist = 0;
    a.step = (uint32_t)step;
    a.v0 = nullptr;
    for (int k = 0; k < 3; ++k) a.v0_all[k] = v0_all ? v0_all[k] : 0.0;
    try {
        run_sample(d, s, a, S.fill);
        MZ_CK(cudaStreamSynchronize(c->stream));
    } catch (...) {
        cudaFree(dF);
        throw;
    }
    cudaFree(dF);
}
