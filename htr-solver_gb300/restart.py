"""Restart directories in HTR's HDF5 layout, through include/htr_restart.h.

`dump` and `load` do what the reference's driver does around a restart:
HDF.dump followed by HDF.write.{timeStep,simTime,SpeciesNames,Versions,
channelForcing} (src/prometeo.rg:1285-1297), and HDF.read.{timeStep,
simTime,channelForcing} followed by HDF.load (src/prometeo.rg:1000-1007).
HDF.dump writes one file per tile of the output partition plus
master.hdf (src/Utils/hdf_helper.rg:933-966); HDF.load checks the master
file's base index space against the grid and reads every tile the master
file lists, whatever the current tiling (src/Utils/hdf_helper.rg:968-1243).
"""
import ctypes as C
import os

from . import abi, runtime

IO_FIELDS = ("rho", "pressure", "temperature", "MolarFracs", "velocity", "dudtBoundary", "dTdtBoundary")
PROFILE_FIELDS = ("MolarFracs_profile", "velocity_profile", "temperature_profile")


def split(fluid, tiles, halo=(0, 0, 0)):
    """Tiles of the whole grid, x fastest, as the reference cuts its output
    partition: the interior (the grid without `halo` ghost layers on each
    side of an axis) in T equal blocks, [k*M//T, (k+1)*M//T) for M interior
    points, the ghost layers joined to the first and last tile
    (scripts/modules/HTRrestart.py:150-161; it asks M % T == 0, where the
    blocks are M/T wide)."""
    n = fluid.shape
    out = []
    for kz in range(tiles[2]):
        for ky in range(tiles[1]):
            for kx in range(tiles[0]):
                k = (kx, ky, kz)
                lo, hi = [], []
                for a in range(3):
                    m = n[a] - 2 * halo[a]
                    lo.append(k[a] * m // tiles[a] + halo[a] - (halo[a] if k[a] == 0 else 0))
                    hi.append((k[a] + 1) * m // tiles[a] - 1 + halo[a] + (halo[a] if k[a] == tiles[a] - 1 else 0))
                out.append(abi.rect(lo, hi))
    return out


def _lib_and_stream(fluid, stream):
    lib = runtime.lib()
    if fluid.device is None:
        return lib, abi.HTR_RESTART_HOST_VIEW, None
    return lib, 0, runtime.stream_handle(stream)


def tile_filename(dirname, rect):
    lib = runtime.lib()
    buf = C.create_string_buffer(4096)
    abi.check(lib, lib.htr_restart_tile_filename(os.fsencode(dirname), rect, buf, len(buf)), "tile file name")
    return os.fsdecode(buf.value)


def dump(dirname, fluid, tiles=(1, 1, 1), time_step=0, sim_time=0.0, channel_forcing=0.0,
         species_names=None, versions=None, profiles=False, stream=None, halo=(0, 0, 0)):
    """Writes the restart fields of `fluid` (host arrays or device tensors)
    as one file per tile (`split`; `halo` = the grid's ghost layers per side
    of each axis gives the reference's tile rectangles and file names) plus
    master.hdf under `dirname`."""
    if fluid.ncells == 0:
        raise abi.HtrError("empty grid")
    os.makedirs(dirname, exist_ok=True)
    lib, flags, s = _lib_and_stream(fluid, stream)
    if profiles:
        flags |= abi.HTR_RESTART_PROFILES
    view = fluid.view()
    if any(t < 1 for t in tiles) or any(tiles[a] > fluid.shape[a] - 2 * halo[a] for a in range(3)):
        raise abi.HtrError(f"cannot cut {fluid.shape} (ghost layers {halo}) into {tiles} tiles")
    parts = split(fluid, tiles, halo)
    d = os.fsencode(dirname)
    for r in parts:
        abi.check(lib, lib.htr_restart_write_tile(d, C.byref(view), r, fluid.nspec, flags, s), "htr_restart_write_tile")
    info = abi.htr_restart_info(int(time_step), float(sim_time), float(channel_forcing))
    t = (C.c_int64 * 3)(*tiles)
    arr = (abi.htr_rect3 * len(parts))(*parts)
    names = None
    if species_names is not None:
        if len(species_names) != fluid.nspec:
            raise abi.HtrError("one species name per species")
        names = (C.c_char_p * fluid.nspec)(*[n.encode() for n in species_names])
    vers = None
    if versions is not None:
        vers = (C.c_char_p * 2)(*[v.encode() for v in versions])
    abi.check(lib, lib.htr_restart_write_master(d, C.byref(info), fluid.bounds(), t, arr, fluid.nspec, names, vers),
              "htr_restart_write_master")
    return parts


def read_master(dirname):
    """The master file's attributes, base index space and tiles."""
    lib = runtime.lib()
    info = abi.htr_restart_info()
    bounds = abi.htr_rect3()
    tiles = (C.c_int64 * 3)()
    d = os.fsencode(dirname)
    abi.check(lib, lib.htr_restart_read_master(d, C.byref(info), C.byref(bounds), tiles, None, 0),
              "htr_restart_read_master")
    n = tiles[0] * tiles[1] * tiles[2]
    parts = (abi.htr_rect3 * n)()
    abi.check(lib, lib.htr_restart_read_master(d, C.byref(info), C.byref(bounds), tiles, parts, n),
              "htr_restart_read_master")
    return {
        "timeStep": info.timeStep, "simTime": info.simTime, "channelForcing": info.channelForcing,
        "bounds": bounds, "tiles": tuple(tiles), "partitions": list(parts),
    }


def check_partitions(dirname, parts, bounds):
    """The master file's tiles lie inside the grid and cover every point of
    it exactly once (a restart with overlapping or missing tiles would leave
    points unloaded or loaded twice)."""
    import numpy as np
    lo = [bounds.lo[i] for i in range(3)]
    ext = [bounds.hi[i] - bounds.lo[i] + 1 for i in range(3)]
    seen = np.zeros((ext[2], ext[1], ext[0]), dtype=np.uint8)
    for r in parts:
        a = [r.lo[i] - lo[i] for i in range(3)]
        b = [r.hi[i] - lo[i] for i in range(3)]
        if any(a[i] < 0 or b[i] >= ext[i] or a[i] > b[i] for i in range(3)):
            raise abi.HtrError(f"{dirname}: tile {list(r.lo)}-{list(r.hi)} lies outside the grid")
        seen[a[2]:b[2] + 1, a[1]:b[1] + 1, a[0]:b[0] + 1] += 1
    if seen.max() > 1:
        raise abi.HtrError(f"{dirname}: tiles overlap")
    if seen.min() < 1:
        raise abi.HtrError(f"{dirname}: tiles leave {int((seen == 0).sum())} grid points uncovered")


def load(dirname, fluid, profiles=False, stream=None, mixture=None):
    """Fills the restart fields of `fluid` from `dirname`; returns the
    master file's timeStep, simTime and channelForcing.  With `mixture` (a
    loaded mixture handle; device grids) the transport properties and the
    conserved variables are then rebuilt from the loaded primitives over the
    whole grid, as a run started from a restart initialises them."""
    if mixture is not None and fluid.device is None:
        raise abi.HtrError("rebuilding the state from a restart needs a device grid")
    m = read_master(dirname)
    b, fb = m["bounds"], fluid.bounds()
    if list(b.lo) != list(fb.lo) or list(b.hi) != list(fb.hi):
        raise abi.HtrError(f"{dirname}: baseIndexSpace {list(b.lo)}-{list(b.hi)} does not match the grid "
                           f"{list(fb.lo)}-{list(fb.hi)}")
    check_partitions(dirname, m["partitions"], fb)
    lib, flags, s = _lib_and_stream(fluid, stream)
    if profiles:
        flags |= abi.HTR_RESTART_PROFILES
    view = fluid.view()
    d = os.fsencode(dirname)
    for r in m["partitions"]:
        abi.check(lib, lib.htr_restart_read_tile(d, C.byref(view), r, fluid.nspec, flags, s), "htr_restart_read_tile")
    if mixture is not None:
        b = fluid.bounds()
        abi.check(lib, lib.htr_UpdatePropertiesFromPrimitive(C.byref(view), b, mixture, s),
                  "htr_UpdatePropertiesFromPrimitive")
        abi.check(lib, lib.htr_UpdateConservedFromPrimitive(C.byref(view), b, mixture, s),
                  "htr_UpdateConservedFromPrimitive")
    return {k: m[k] for k in ("timeStep", "simTime", "channelForcing")}
