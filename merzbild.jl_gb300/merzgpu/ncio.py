"""netCDF output of cell and surface properties, mirroring io.jl.

``NCDataHolder`` / ``NCDataHolderSurf`` / ``write_netcdf`` / ``close_netcdf``
keep the reference's signatures (io.jl:116-330, :430-603).  The file is
written by libmerzgpu (netCDF classic, 64-bit offset container; see
include/merzgpu.h for the two differences from the reference's netCDF-4
files).  Writing a device property set (:class:`PhysProps`,
:class:`SurfProps`) enqueues the record on the device stream; the library's
writer thread puts it in the file, so the time loop does not wait for the
disk.  Host property sets (:class:`HostPhysProps`, :class:`HostSurfProps`, or
the dicts returned by ``fetch()``) are written from host memory.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from ._lib import MerzError, lib, ptr

_PROPS_NAMES = ("length_particle_array", "moments", "np", "nparticles", "ndens", "v", "T")
_SURF_NAMES = ("np", "nparticles", "fluxes", "force", "normal_pressure", "shear_pressure", "kinetic_energy_flux")


class IOSkipList:
    """IOSkipList(list_of_variables_to_skip) (io.jl:19-80)."""

    def __init__(self, list_of_variables_to_skip=()):
        s = list(list_of_variables_to_skip)
        self.names = s
        self.skip_length_particle_array = "length_particle_array" in s
        self.skip_moments = "moments" in s
        self.skip_number_of_particles = "np" in s or "nparticles" in s
        self.skip_number_density = "ndens" in s
        self.skip_velocity = "v" in s
        self.skip_temperature = "T" in s


class IOSkipListSurf:
    """IOSkipListSurf(list_of_variables_to_skip) (io.jl:334-418)."""

    def __init__(self, list_of_variables_to_skip=()):
        s = list(list_of_variables_to_skip)
        self.names = s
        self.skip_number_of_particles = "np" in s or "nparticles" in s
        self.skip_fluxes = "fluxes" in s
        self.skip_force = "force" in s
        self.skip_normal_pressure = "normal_pressure" in s
        self.skip_shear_pressure = "shear_pressure" in s
        self.skip_kinetic_energy_flux = "kinetic_energy_flux" in s


class HostPhysProps:
    """PhysProps(n_cells, n_species, moments_list; Tref, ndens_not_Np) held in
    host memory (physical_props.jl:24-58), for writing arrays computed
    elsewhere.  Shapes as the reference: np, n, T (cells, species); v (3,
    cells, species); moments (n_moments, cells, species); lpa (species)."""

    def __init__(self, n_cells, n_species, moments_list=(), Tref=300.0, ndens_not_Np=False):
        self.n_cells, self.n_species = int(n_cells), int(n_species)
        self.moment_powers = list(moments_list)
        self.n_moments = len(self.moment_powers)
        self.Tref = Tref
        self.ndens_not_Np = bool(ndens_not_Np)
        self.lpa = np.zeros(self.n_species)
        self.np = np.zeros((self.n_cells, self.n_species))
        self.n = np.zeros((self.n_cells, self.n_species))
        self.v = np.zeros((3, self.n_cells, self.n_species))
        self.T = np.zeros((self.n_cells, self.n_species))
        self.moments = np.zeros((self.n_moments, self.n_cells, self.n_species))


class HostSurfProps:
    """SurfProps in host memory (surface_props.jl:22-67): (elements, species)
    arrays, force and shear_pressure (3, elements, species)."""

    def __init__(self, n_elements, n_species):
        self.n_elements, self.n_species = int(n_elements), int(n_species)
        shp, shp3 = (self.n_elements, self.n_species), (3, self.n_elements, self.n_species)
        self.np = np.zeros(shp)
        self.flux_incident = np.zeros(shp)
        self.flux_reflected = np.zeros(shp)
        self.force = np.zeros(shp3)
        self.normal_pressure = np.zeros(shp)
        self.shear_pressure = np.zeros(shp3)
        self.kinetic_energy_flux = np.zeros(shp)


def _colmajor(a):
    """Flatten an array in Julia (column-major) order, as the file's record slab."""
    return np.ascontiguousarray(np.asarray(a, np.float64).ravel(order="F"))


def _attrs(global_attributes):
    keep = []
    items = list((global_attributes or {}).items())
    arr = (L.NcAttribute * max(1, len(items)))()
    for k, (name, val) in enumerate(items):
        nb = str(name).encode()
        if isinstance(val, str):
            buf = val.encode()
            data = C.create_string_buffer(buf, len(buf))
            t, cnt = 0, len(buf)
        else:
            a = np.atleast_1d(np.asarray(val))
            if np.issubdtype(a.dtype, np.integer):
                data = np.ascontiguousarray(a, np.int32)
                t = 1
            else:
                data = np.ascontiguousarray(a, np.float64)
                t = 2
            cnt = data.size
        keep += [nb, data]
        addr = C.addressof(data) if isinstance(data, C.Array) else data.ctypes.data
        arr[k] = L.NcAttribute(nb, t, cnt, addr)
    return arr, len(items), keep


def _names(names):
    enc = [str(n).encode() for n in names]
    arr = (C.c_char_p * max(1, len(enc)))(*enc)
    return arr, len(enc), enc


class _NCFile:
    def __init__(self):
        self.h = C.c_void_p()
        self._ctx = None

    def _ck(self, rc):
        if rc != L.MZ_OK:
            buf = C.create_string_buffer(1024)
            if self.h:
                lib().mz_nc_last_error(self.h, buf, 1024)
            raise MerzError(rc, buf.value.decode(errors="replace"))

    def flush(self):
        self._ck(lib().mz_nc_flush(self.h))

    def records(self):
        n = C.c_int64()
        self._ck(lib().mz_nc_records(self.h, C.byref(n)))
        return n.value

    def close(self):
        if self.h:
            h, self.h = self.h, C.c_void_p()
            rc = lib().mz_nc_close(h)
            if rc != L.MZ_OK:
                raise MerzError(rc, "netCDF file could not be completed")

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _create_err(rc, ctx):
    msg = ""
    if ctx is not None and ctx.h:
        buf = C.create_string_buffer(1024)
        lib().mz_last_error(ctx.h, buf, 1024)
        msg = buf.value.decode(errors="replace")
    raise MerzError(rc, msg or "netCDF file could not be created")


class NCDataHolder(_NCFile):
    """NCDataHolder(nc_filename, [names_skip_list,] species_data, phys_props;
    global_attributes) (io.jl:143-243).  phys_props is a device
    :class:`PhysProps` (records are then written from the device) or a
    :class:`HostPhysProps`."""

    def __init__(self, nc_filename, *args, global_attributes=None):
        super().__init__()
        if len(args) == 2:
            names_skip_list, (species_data, phys_props) = [], args
        else:
            names_skip_list, species_data, phys_props = args
        self.skip_list = IOSkipList(names_skip_list)
        self.ndens_not_Np = bool(phys_props.ndens_not_Np)
        dom = getattr(phys_props, "domain", None)
        self._ctx = dom.ctx if dom is not None else None
        n_cells = dom.n_cells if dom is not None else phys_props.n_cells
        n_species = dom.n_species if dom is not None else phys_props.n_species
        powers = np.ascontiguousarray(phys_props.moment_powers, np.int32)
        skip, nsk, k1 = _names(names_skip_list)
        spn, ns, k2 = _names([s.name for s in species_data])
        att, na, k3 = _attrs(global_attributes)
        rc = lib().mz_nc_props_create(str(nc_filename).encode(), skip, nsk, spn, ns, n_species, n_cells, len(powers),
                                      ptr(powers, C.c_int32) if len(powers) else None, int(self.ndens_not_Np), att,
                                      na, self._ctx.h if self._ctx is not None else None, C.byref(self.h))
        if rc != L.MZ_OK:
            _create_err(rc, self._ctx)


class NCDataHolderSurf(_NCFile):
    """NCDataHolderSurf(nc_filename, [names_skip_list,] species_data,
    surf_props; global_attributes) (io.jl:457-547)."""

    def __init__(self, nc_filename, *args, global_attributes=None):
        super().__init__()
        if len(args) == 2:
            names_skip_list, (species_data, surf_props) = [], args
        else:
            names_skip_list, species_data, surf_props = args
        self.skip_list = IOSkipListSurf(names_skip_list)
        dom = getattr(surf_props, "domain", None)
        self._ctx = dom.ctx if dom is not None else None
        n_elements = 2 if dom is not None else surf_props.n_elements
        n_species = dom.n_species if dom is not None else surf_props.n_species
        skip, nsk, k1 = _names(names_skip_list)
        spn, ns, k2 = _names([s.name for s in species_data])
        att, na, k3 = _attrs(global_attributes)
        rc = lib().mz_nc_surf_create(str(nc_filename).encode(), skip, nsk, spn, ns, n_species, n_elements, att, na,
                                     self._ctx.h if self._ctx is not None else None, C.byref(self.h))
        if rc != L.MZ_OK:
            _create_err(rc, self._ctx)


def write_netcdf(ds, props, timestep, sync_freq=0):
    """write_netcdf(ds, phys_props | surf_props, timestep; sync_freq)
    (io.jl:274-317, :566-603).  Raises MerzError (code MZ_E_ARG) when a cell
    property set's ndens_not_Np differs from the file's, like the reference's
    ErrorException."""
    from .api import PhysProps, SurfProps

    if isinstance(ds, NCDataHolder):
        if isinstance(props, PhysProps):
            ds._ck(lib().mz_nc_props_write(ds.h, props.h, float(timestep), int(sync_freq)))
            return
        g = props if isinstance(props, dict) else vars(props)
        nd = int(bool(g.get("ndens_not_Np", ds.ndens_not_Np)))
        a = {k: _colmajor(g[k]) if g.get(k) is not None else None for k in ("lpa", "np", "n", "v", "T", "moments")}
        ds._ck(lib().mz_nc_props_write_host(ds.h, ptr(a["lpa"]), ptr(a["np"]), ptr(a["n"]), ptr(a["v"]), ptr(a["T"]),
                                            ptr(a["moments"]), nd, float(timestep), int(sync_freq)))
    elif isinstance(ds, NCDataHolderSurf):
        if isinstance(props, SurfProps):
            ds._ck(lib().mz_nc_surf_write(ds.h, props.h, float(timestep), int(sync_freq)))
            return
        g = props if isinstance(props, dict) else vars(props)
        keys = ("np", "flux_incident", "flux_reflected", "force", "normal_pressure", "shear_pressure",
                "kinetic_energy_flux")
        a = [_colmajor(g[k]) if g.get(k) is not None else None for k in keys]
        ds._ck(lib().mz_nc_surf_write_host(ds.h, *[ptr(x) for x in a], float(timestep), int(sync_freq)))
    else:
        raise TypeError("write_netcdf: not a netCDF data holder")


def close_netcdf(ds):
    """close_netcdf(ds) (io.jl:251-253)."""
    ds.close()


__all__ = ["IOSkipList", "IOSkipListSurf", "HostPhysProps", "HostSurfProps", "NCDataHolder", "NCDataHolderSurf",
           "write_netcdf", "close_netcdf"]
