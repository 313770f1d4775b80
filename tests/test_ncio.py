"""netCDF output written from host arrays (no GPU needed): the reference's I/O
tests test/test_io.jl and test/test_io_surf.jl, read back with an
independent reader (scipy's netCDF classic reader), plus the container's
layout: dimension order, types, species names, attributes, record count."""
import os
import struct

import numpy as np
import pytest

import merzgpu as mz

netcdf = pytest.importorskip("scipy.io").netcdf_file
EPS = np.finfo(float).eps


@pytest.fixture(scope="module", autouse=True)
def built():
    from merzgpu import build as b

    b.build()


def _read(path):
    f = netcdf(path, "r", mmap=False)
    out = {k: v.data.copy() for k, v in f.variables.items()}
    dims = dict(f.dimensions)
    vdims = {k: v.dimensions for k, v in f.variables.items()}
    att = dict(f._attributes)
    f.close()
    return out, dims, vdims, att


def test_skip_lists_match_the_reference():
    # test/test_io.jl:4-30 and test/test_io_surf.jl:56-82
    s = mz.IOSkipList()
    assert not any((s.skip_length_particle_array, s.skip_moments, s.skip_number_of_particles,
                    s.skip_number_density, s.skip_velocity, s.skip_temperature))
    s = mz.IOSkipList(["length_particle_array", "ndens", "v"])
    assert (s.skip_length_particle_array, s.skip_moments, s.skip_number_of_particles, s.skip_number_density,
            s.skip_velocity, s.skip_temperature) == (True, False, False, True, True, False)
    s = mz.IOSkipList(["T", "np"])
    assert (s.skip_length_particle_array, s.skip_moments, s.skip_number_of_particles, s.skip_number_density,
            s.skip_velocity, s.skip_temperature) == (False, False, True, False, False, True)
    s = mz.IOSkipListSurf(["np", "force", "shear_pressure"])
    assert (s.skip_number_of_particles, s.skip_fluxes, s.skip_force, s.skip_normal_pressure,
            s.skip_shear_pressure, s.skip_kinetic_energy_flux) == (True, False, True, False, True, False)
    s = mz.IOSkipListSurf(["fluxes", "normal_pressure", "kinetic_energy_flux"])
    assert (s.skip_number_of_particles, s.skip_fluxes, s.skip_force, s.skip_normal_pressure,
            s.skip_shear_pressure, s.skip_kinetic_energy_flux) == (False, True, False, True, False, True)


def test_props_file_with_skip_list(tmp_path):
    # test/test_io.jl:32-75: 4 cells, 2 species, no moments, three records
    sp = [mz.Species("Ar", mz.AR_MASS)]
    pp = mz.HostPhysProps(4, 2, [], Tref=1)
    assert pp.ndens_not_Np is False
    path = str(tmp_path / "tmp_skiplist.nc")
    skip = ["T", "np"]
    ds = mz.NCDataHolder(path, skip, sp, pp)
    assert ds.ndens_not_Np is False
    pp.T[:] = -100.0
    pp.n[:] = -100.0
    pp.np[:] = -100.0
    pp.lpa[:] = 30.0
    pp.v[:] = 30.0
    for t in (0, 1, 2):
        mz.write_netcdf(ds, pp, t)
    mz.close_netcdf(ds)
    out, dims, vdims, att = _read(path)
    for name in skip:
        assert name not in out
    for name in ("v", "ndens", "length_particle_array"):
        assert name in out
    # Julia sizes (3, 4, 2, 3), (4, 2, 3), (2, 3) are the reverse of the file's
    assert out["v"].shape == (3, 2, 4, 3)
    assert out["ndens"].shape == (3, 2, 4)
    assert out["length_particle_array"].shape == (3, 2)
    assert vdims["v"] == ("timestep", "n_species", "n_cells", "vel_components")
    assert np.all(out["v"] == 30.0) and np.all(out["ndens"] == -100.0)
    assert np.array_equal(out["timestep"], [0.0, 1.0, 2.0])
    assert att["COMMENT ndens"].decode().startswith("In this file, the ndens variable stores # of physical")
    assert "moments" not in out and "n_moments" not in dims  # no moments: no zero-length dimension


def test_props_file_rejects_the_other_ndens_kind(tmp_path):
    # test/test_io.jl:77-95
    sp = [mz.Species("Ar", mz.AR_MASS)]
    pp_nd = mz.HostPhysProps(4, 2, [], Tref=1, ndens_not_Np=True)
    pp = mz.HostPhysProps(4, 2, [], Tref=1)
    path = str(tmp_path / "tmp_ndens.nc")
    ds = mz.NCDataHolder(path, [], sp, pp_nd)
    assert ds.ndens_not_Np is True
    with pytest.raises(mz.MerzError) as e:
        mz.write_netcdf(ds, pp, 0)
    assert "Inconsistent computation of ndens" in str(e.value)
    mz.close_netcdf(ds)
    out, _, _, att = _read(path)
    assert out["timestep"].shape == (0,)
    assert att["COMMENT ndens"].decode().startswith("In this file, the ndens variable stores the number density")


def test_props_file_values_and_layout(tmp_path):
    """Every variable of a file with moments round-trips exactly, in the
    reference's column-major layout; species names, moment powers and
    global attributes as given."""
    rng = np.random.default_rng(5)
    sp = [mz.Species("Ar", mz.AR_MASS), mz.Species("He", mz.HE_MASS)]
    nc, ns = 7, 2
    pp = mz.HostPhysProps(nc, ns, [4, 6, 8], Tref=273.0)
    path = str(tmp_path / "props.nc")
    ds = mz.NCDataHolder(path, sp, pp, global_attributes={"case": "couette", "nx": 7, "L": 5e-4})
    written = []
    for t in range(5):
        for k in ("np", "n", "v", "T", "moments", "lpa"):
            getattr(pp, k)[...] = rng.normal(size=getattr(pp, k).shape)
        written.append({k: getattr(pp, k).copy() for k in ("np", "n", "v", "T", "moments", "lpa")})
        mz.write_netcdf(ds, pp, 10 * t, sync_freq=2)
    ds.flush()
    assert ds.records() == 5
    mz.close_netcdf(ds)
    out, dims, vdims, att = _read(path)
    assert dims == {"vel_components": 3, "n_cells": nc, "n_species": ns, "n_moments": 3, "timestep": None,
                    "species_name_length": 2}
    assert np.array_equal(out["timestep"], [0, 10, 20, 30, 40])
    assert out["moment_powers"].dtype == np.dtype(">i4") and list(out["moment_powers"]) == [4, 6, 8]
    assert [b"".join(r).rstrip(b"\0").decode() for r in out["species_names"]] == ["Ar", "He"]
    assert att["case"] == b"couette" and int(att["nx"]) == 7 and float(att["L"]) == 5e-4
    for t, w in enumerate(written):
        # file order (timestep, species, cells, ...) = transpose of the Julia order
        assert np.array_equal(out["np"][t], w["np"].T)
        assert np.array_equal(out["ndens"][t], w["n"].T)
        assert np.array_equal(out["T"][t], w["T"].T)
        assert np.array_equal(out["v"][t], w["v"].transpose(2, 1, 0))
        assert np.array_equal(out["moments"][t], w["moments"].transpose(2, 1, 0))
        assert np.array_equal(out["length_particle_array"][t], w["lpa"])
    with open(path, "rb") as f:
        head = f.read(8)
    assert head[:4] == b"CDF\x02" and struct.unpack(">I", head[4:])[0] == 5


def _set_surf_data(sp, t):
    # test/test_io_surf.jl:3-35
    sp.np[0, 0], sp.np[1, 0] = 1.0 * t, 2.0 * t
    sp.flux_incident[0, 0], sp.flux_incident[1, 0] = 2.0 * t, 3.0 * t
    sp.flux_reflected[0, 0], sp.flux_reflected[1, 0] = 4.0 * t, 5.0 * t
    sp.force[:, 0, 0] = (10.0 * t, 11.0 * t, 12.0 * t)
    sp.force[:, 1, 0] = (20.0 * t, 21.0 * t, 22.0 * t)
    sp.normal_pressure[0, 0], sp.normal_pressure[1, 0] = 22.0 * t, 25.0 * t
    sp.shear_pressure[:, 0, 0] = (40.0 * t, 41.0 * t, 42.0 * t)
    sp.shear_pressure[:, 1, 0] = (30.0 * t, 31.0 * t, 32.0 * t)
    sp.kinetic_energy_flux[0, 0], sp.kinetic_energy_flux[1, 0] = 27.0 * t, 29.0 * t


def test_surface_file_matches_the_reference_test(tmp_path):
    # test/test_io_surf.jl:84-122
    sp = [mz.Species("Ar", mz.AR_MASS)]
    surf = mz.HostSurfProps(2, 1)
    path = str(tmp_path / "tmp_no_skiplist.nc")
    ds = mz.NCDataHolderSurf(path, [], sp, surf)
    _set_surf_data(surf, 0)
    mz.write_netcdf(ds, surf, 0)
    _set_surf_data(surf, 1)
    mz.write_netcdf(ds, surf, 1, sync_freq=1)
    _set_surf_data(surf, 2)
    mz.write_netcdf(ds, surf, 2)
    mz.close_netcdf(ds)
    out, _, vdims, _ = _read(path)
    for name in ("np", "flux_incident", "flux_reflected", "force", "normal_pressure", "shear_pressure",
                 "kinetic_energy_flux"):
        assert name in out
    for name in ("np", "flux_incident", "flux_reflected", "normal_pressure", "kinetic_energy_flux"):
        assert out[name].shape == (3, 1, 2)  # Julia (2, 1, 3)
    assert out["force"].shape == (3, 1, 2, 3) and out["shear_pressure"].shape == (3, 1, 2, 3)
    assert vdims["force"] == ("timestep", "n_species", "n_elements", "vector_components")
    ref = mz.HostSurfProps(2, 1)
    for t in range(3):
        _set_surf_data(ref, t)
        for name in ("np", "flux_incident", "flux_reflected", "normal_pressure", "kinetic_energy_flux"):
            assert np.max(np.abs(getattr(ref, name).T - out[name][t])) < 2 * EPS
        for name in ("force", "shear_pressure"):
            assert np.max(np.abs(getattr(ref, name).transpose(2, 1, 0) - out[name][t])) < 2 * EPS


def test_surface_file_with_skip_list(tmp_path):
    # test/test_io_surf.jl:125-146
    sp = [mz.Species("Ar", mz.AR_MASS)]
    surf = mz.HostSurfProps(2, 1)
    path = str(tmp_path / "tmp_skiplist.nc")
    skip = ["np", "force", "shear_pressure"]
    ds = mz.NCDataHolderSurf(path, skip, sp, surf)
    _set_surf_data(surf, 0)
    mz.write_netcdf(ds, surf, 0)
    mz.close_netcdf(ds)
    out, _, _, _ = _read(path)
    for name in skip:
        assert name not in out
    for name in ("flux_incident", "flux_reflected", "normal_pressure", "kinetic_energy_flux"):
        assert name in out


def test_unwritable_path_reports_an_error(tmp_path):
    sp = [mz.Species("Ar", mz.AR_MASS)]
    with pytest.raises(mz.MerzError):
        mz.NCDataHolder(str(tmp_path / "no_such_dir" / "x.nc"), sp, mz.HostPhysProps(2, 1))
