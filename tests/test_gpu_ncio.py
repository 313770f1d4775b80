"""Time-averaged output written from the device (write_netcdf of device
property sets, io.jl:274-317 and :566-603): the Couette loop of
simulations/1D/couette_benchmarking.jl writing averaged cell and surface
properties every few steps while the next steps run.  The file's records
equal the sets' contents at the write points (bit for bit for cell
properties), and the last averaged record equals the oracle's time loop."""
import numpy as np
import pytest

import merzgpu as mz
from test_gpu_step import couette_plan, couette_setup, oracle_couette

pytestmark = pytest.mark.gpu

netcdf = pytest.importorskip("scipy.io").netcdf_file


@pytest.fixture(scope="module")
def ctx():
    import merzgpu.build as b

    b.build()
    c = mz.Context(0)
    yield c
    c.close()


CHUNK, CHUNKS, AVG_FROM = 3, 4, 4  # steps 1-3 not averaged, 4-12 averaged


def _run(ctx, orc, tmp_path, write):
    sp, grid, walls, dt, o, dom, seed = couette_setup(ctx, orc, nx=40, ppc=100, seed=41)
    inst, avg = mz.PhysProps(dom), mz.PhysProps(dom)
    s_inst, s_avg = mz.SurfProps(dom), mz.SurfProps(dom)
    dom.set_step_surface(s_inst, s_avg)
    n_avg = CHUNK * CHUNKS - AVG_FROM + 1
    files = None
    if write:
        files = (mz.NCDataHolder(str(tmp_path / "avg.nc"), sp, avg, global_attributes={"n_avg": n_avg}),
                 mz.NCDataHolder(str(tmp_path / "inst.nc"), ["length_particle_array"], sp, inst),
                 mz.NCDataHolderSurf(str(tmp_path / "surf_avg.nc"), sp, s_avg))
    fetched = []
    for k in range(CHUNKS):
        plan = couette_plan(grid, walls, dt, step0=k * CHUNK, avg_start=0 if k == 0 else 1, n_avg=n_avg)
        dom.step(plan, CHUNK, inst, avg)
        t = (k + 1) * CHUNK
        if write:
            # enqueued behind the steps; the next chunk starts without waiting
            mz.write_netcdf(files[0], avg, t)
            mz.write_netcdf(files[1], inst, t, sync_freq=2)
            mz.write_netcdf(files[2], s_avg, t)
        else:
            fetched.append((avg.fetch(), inst.fetch(), s_avg.fetch()))
    if write:
        for f in files:
            mz.close_netcdf(f)
    return fetched, (sp, grid, walls, dt, o, seed)


def _read(path):
    f = netcdf(path, "r", mmap=False)
    out = {k: v.data.copy() for k, v in f.variables.items()}
    f.close()
    return out


def test_device_output_records_equal_the_sets(ctx, orc, tmp_path):
    _run(ctx, orc, tmp_path, write=True)
    fetched, (sp, grid, walls, dt, o, seed) = _run(ctx, orc, tmp_path, write=False)
    fa, fi, fs = _read(str(tmp_path / "avg.nc")), _read(str(tmp_path / "inst.nc")), _read(str(tmp_path / "surf_avg.nc"))
    times = [CHUNK * (k + 1) for k in range(CHUNKS)]
    for f in (fa, fi, fs):
        assert np.array_equal(f["timestep"], times)
    assert "length_particle_array" not in fi and "length_particle_array" in fa
    for k, (a, i, s) in enumerate(fetched):
        for f, r in ((fa, a), (fi, i)):
            assert np.array_equal(f["np"][k], r["np"].T)
            assert np.array_equal(f["ndens"][k], r["n"].T)
            assert np.array_equal(f["T"][k], r["T"].T)
            assert np.array_equal(f["v"][k], r["v"].transpose(2, 1, 0))
        assert np.array_equal(fa["length_particle_array"][k], a["lpa"])
        # wall sums are atomic additions: equal to round-off between runs
        for name in ("np", "flux_incident", "flux_reflected", "normal_pressure", "kinetic_energy_flux"):
            ref = s[name].T
            assert np.allclose(fs[name][k], ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max()), name
        for name in ("force", "shear_pressure"):
            ref = s[name].transpose(2, 1, 0)
            assert np.allclose(fs[name][k], ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max()), name
    assert np.all(fa["np"][0] == 0.0) and np.all(fa["np"][1] > 0.0)  # averaging starts at step 4
    # the last averaged record is the oracle loop's time average
    ref_avg = oracle_couette(orc, o, grid, walls, dt, seed, CHUNK * CHUNKS, AVG_FROM)
    last = {k: v[-1] for k, v in fa.items()}
    assert np.allclose(last["np"][0], ref_avg[0], rtol=1e-14, atol=0)
    assert np.allclose(last["T"][0], ref_avg[5], rtol=1e-11, atol=0)
    vscale = np.abs(ref_avg[2:5]).max()
    assert np.allclose(last["v"][0].T, ref_avg[2:5], rtol=0, atol=1e-11 * vscale)
