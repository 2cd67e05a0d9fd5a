"""Restart files in the reference's HDF5 layout (include/htr_restart.h).

The oracle is an independent HDF5 reader (oracle/h5read.py).  Both it and
the library's reader are pinned against a file libhdf5 wrote (a MATLAB 7.3
file among scipy's test data, with its 512-byte user block): its dataset
`testdouble` is 0:pi/4:2*pi with attribute MATLAB_class = "double".  The
writer is checked structure by structure against that file (datatype and
fill-value messages byte for byte, superblock and group-node parameters,
the local heap's free-list convention) and field by field through the
oracle.  The layout itself follows the reference's writer: tile file names
(src/Utils/hdf_helper.rg:357-367), one (z, y, x) dataset per restart field
with vector fields as arrays of doubles (:199-331), the master file's
attributes and partitions (:845-931, :1245-1431).
"""
import ctypes as C
import glob
import os
import shutil

import numpy as np
import pytest

from htr_gb300 import abi, fluid, restart, runtime

from oracle import h5read

MAT = None
try:
    import scipy.io.matlab as _m
    _cand = os.path.join(os.path.dirname(_m.__file__), "tests", "data", "testhdf5_7.4_GLNX86.mat")
    MAT = _cand if os.path.exists(_cand) else None
except Exception:
    MAT = None

needs_lib = pytest.mark.skipif(not os.path.exists(runtime.LIB_PATH), reason="CUDA library not built")
needs_mat = pytest.mark.skipif(MAT is None, reason="no libhdf5-written file available")

SPECIES = ["N2", "O2", "NO", "N", "O"]


def random_fluid(shape, nspec=5, seed=0, profiles=False, device=None):
    f = fluid.Fluid(shape, nspec)
    rng = np.random.default_rng(seed)
    names = restart.IO_FIELDS + (restart.PROFILE_FIELDS if profiles else ())
    for n in names:
        f[n] = rng.standard_normal(f[n].shape)
    return f if device is None else f.to_device(device)


def tile_slice(a, r):
    return a[r.lo[2]:r.hi[2] + 1, r.lo[1]:r.hi[1] + 1, r.lo[0]:r.hi[0] + 1]


# ---------------------------------------------------------------- pinning

@needs_mat
def test_oracle_reads_a_libhdf5_file():
    f = h5read.File(MAT)
    assert f.sb_at == 512  # after the MATLAB user block
    a, attrs = f.datasets["testdouble"]
    assert a.dtype == np.float64 and a.shape == (9, 1)
    np.testing.assert_allclose(a.ravel(), np.arange(9) * np.pi / 4, rtol=1e-15, atol=0)
    assert attrs["MATLAB_class"] == b"double"
    # libhdf5's group parameters and the local heap's free-list end marker
    assert (f.leaf_k, f.internal_k) == (4, 16)
    heap = f._heap(f.root_heap)
    head = f.heap_free_head
    assert int.from_bytes(heap[head:head + 8], "little") == 1


@needs_mat
@needs_lib
def test_library_reads_a_libhdf5_file():
    lib = runtime.lib()
    rank, dims, per = C.c_int(), (C.c_int64 * 8)(), C.c_int64()
    abi.check(lib, lib.htr_h5_dataset_shape(MAT.encode(), b"testdouble", C.byref(rank), dims, C.byref(per)))
    assert rank.value == 2 and list(dims[:2]) == [9, 1] and per.value == 1
    out = (C.c_double * 9)()
    abi.check(lib, lib.htr_h5_read_doubles(MAT.encode(), b"testdouble", out, 9))
    ref = h5read.File(MAT).datasets["testdouble"][0].ravel()
    assert np.array_equal(np.frombuffer(out, dtype=np.float64), ref)
    s = C.create_string_buffer(32)
    abi.check(lib, lib.htr_h5_string_attribute(MAT.encode(), b"testdouble", b"MATLAB_class", 0, s, 32))
    assert s.value == b"double"
    assert lib.htr_h5_read_doubles(MAT.encode(), b"testdouble", out, 8) == abi.HTR_ERR_ARGUMENT
    assert lib.htr_h5_read_doubles(MAT.encode(), b"nothing", out, 9) == abi.HTR_ERR_FORMAT


@needs_mat
@needs_lib
def test_writer_structures_match_libhdf5(tmp_path):
    real = h5read.File(MAT)
    f = random_fluid((5, 4, 3))
    restart.dump(str(tmp_path), f)
    path = glob.glob(str(tmp_path / "*-*.hdf"))[0]
    ours = h5read.File(path)
    msgs = {t: (fl, b) for t, fl, b in ours.messages["rho"]}
    theirs = {t: (fl, b) for t, fl, b in real.messages["testdouble"]}
    assert msgs[0x03] == theirs[0x03]  # IEEE binary64 little-endian datatype
    assert msgs[0x05] == theirs[0x05]  # fill value message
    assert (ours.leaf_k, ours.internal_k, ours.so, ours.sl) == (real.leaf_k, real.internal_k, real.so, real.sl)
    heap = ours._heap(ours.root_heap)
    assert int.from_bytes(heap[ours.heap_free_head:ours.heap_free_head + 8], "little") == 1
    raw = open(path, "rb").read()
    assert raw[:8] == h5read.SIGNATURE and ours.eof == len(raw)
    assert raw[8:16] == real.b[real.sb_at + 8:real.sb_at + 16]  # versions, sizes
    # the layout message: version 3, contiguous, 8-byte aligned data
    lay = msgs[0x08][1]
    assert lay[0] == 3 and lay[1] == 1 and int.from_bytes(lay[2:10], "little") % 8 == 0


# ---------------------------------------------------------------- layout

@needs_lib
def test_tile_filename():
    assert restart.tile_filename("d", abi.rect((0, 0, 0), (9, 19, 29))) == "d/0,0,0-9,19,29.hdf"
    assert restart.tile_filename("a/b", abi.rect((-3, 4, 5), (1 << 40, 7, 8))) == \
        f"a/b/-3,4,5-{1 << 40},7,8.hdf"


@needs_lib
@pytest.mark.parametrize("tiles,profiles", [((1, 1, 1), False), ((2, 1, 2), True), ((3, 2, 1), False)])
def test_restart_round_trip_host(tmp_path, tiles, profiles):
    f = random_fluid((7, 5, 4), seed=3, profiles=profiles)
    parts = restart.dump(str(tmp_path), f, tiles=tiles, time_step=4711, sim_time=0.125,
                         channel_forcing=-2.5, species_names=SPECIES, versions=["1.2.3-abc", "legion-x"],
                         profiles=profiles)
    names = restart.IO_FIELDS + (restart.PROFILE_FIELDS if profiles else ())
    # every tile file, read by the oracle, holds the tile's slice of each field
    files = sorted(os.listdir(tmp_path))
    assert len(files) == len(parts) + 1 and "master.hdf" in files
    covered = np.zeros((4, 5, 7), dtype=int)
    for r in parts:
        t = h5read.File(restart.tile_filename(str(tmp_path), r))
        assert sorted(t.datasets) == sorted(names)
        for n in names:
            a, _ = t.datasets[n]
            assert a.dtype == np.float64
            assert np.array_equal(a, tile_slice(f[n], r)), n
        tile_slice(covered, r)[...] += 1
    assert (covered == 1).all()
    # master file: attributes and partitions as the reference writes them
    m = h5read.File(str(tmp_path / "master.hdf"))
    assert m.attrs["IO_VERSION"] == b"1.0.0" and m.attrs["IO_VERSION"].dtype.itemsize == 8
    assert m.attrs["timeStep"].dtype == np.dtype("<i4") and int(m.attrs["timeStep"]) == 4711
    assert float(m.attrs["simTime"]) == 0.125 and float(m.attrs["channelForcing"]) == -2.5
    b = m.attrs["baseIndexSpace"]
    assert b["lo"].item() == (0, 0, 0) and b["hi"].item() == (6, 4, 3)
    assert m.attrs["tilesNumber"].item() == tiles
    assert list(m.attrs["SpeciesNames"]) == [s.encode() for s in SPECIES]
    assert m.attrs["SpeciesNames"].dtype.itemsize == 21
    assert list(m.attrs["Versions"]) == [b"1.2.3-abc", b"legion-x"]
    p, _ = m.datasets["partitions"]
    assert p.shape == (tiles[2], tiles[1], tiles[0])
    for k, r in enumerate(parts):
        x, y, z = k % tiles[0], k // tiles[0] % tiles[1], k // (tiles[0] * tiles[1])
        assert tuple(p[z, y, x]["lo"]) == tuple(r.lo) and tuple(p[z, y, x]["hi"]) == tuple(r.hi)
    # load into a zeroed state: restart fields restored bit for bit
    g = fluid.Fluid(f.shape, f.nspec)
    info = restart.load(str(tmp_path), g, profiles=profiles)
    assert info == {"timeStep": 4711, "simTime": 0.125, "channelForcing": -2.5}
    for n in names:
        assert np.array_equal(g[n], f[n]), n
    assert not g["Conserved"].any()  # not a restart field


def test_tiles_follow_the_reference_partition():
    """With the ghost layers given, the tiles are the reference's: equal
    interior blocks, ghosts joined to the outer tiles (the rule of
    scripts/modules/HTRrestart.py:130-161, written out here)."""
    f = fluid.Fluid((514, 194, 128), 5, fields=["rho"])  # 512 x 192 x 128 interior, ghosts in x and y
    tiles, halo = (4, 2, 2), (1, 1, 0)
    got = restart.split(f, tiles, halo)
    nt = [512 // 4, 192 // 2, 128 // 2]
    k = 0
    for z in range(tiles[2]):
        for y in range(tiles[1]):
            for x in range(tiles[0]):
                c = (x, y, z)
                lo = [c[a] * nt[a] + halo[a] for a in range(3)]
                hi = [(c[a] + 1) * nt[a] - 1 + halo[a] for a in range(3)]
                for a in range(3):
                    if c[a] == 0:
                        lo[a] -= halo[a]
                    if c[a] == tiles[a] - 1:
                        hi[a] += halo[a]
                assert list(got[k].lo) == lo and list(got[k].hi) == hi, (c, list(got[k].lo), list(got[k].hi))
                k += 1
    # without ghost layers: blocks of the whole grid
    assert [list(r.hi) for r in restart.split(fluid.Fluid((6, 4, 2), 1, fields=["rho"]), (2, 1, 1))] == \
        [[2, 3, 1], [5, 3, 1]]


@needs_lib
def test_load_reads_the_tiling_of_the_master_file(tmp_path):
    f = random_fluid((8, 6, 5), seed=4)
    restart.dump(str(tmp_path), f, tiles=(2, 3, 1), halo=(1, 0, 1))
    g = fluid.Fluid(f.shape, f.nspec)
    restart.load(str(tmp_path), g)
    for n in restart.IO_FIELDS:
        assert np.array_equal(g[n], f[n])
    m = restart.read_master(str(tmp_path))
    assert m["tiles"] == (2, 3, 1) and len(m["partitions"]) == 6


@needs_lib
def test_strided_views(tmp_path):
    """Fields that are slices of larger arrays (non-dense strides)."""
    big = random_fluid((9, 7, 6), seed=5)
    f = fluid.Fluid((4, 3, 2), 5)
    for n in restart.IO_FIELDS:
        f.arrays[n] = big[n][1:5:2, 2:5, 1:9:2]
    restart.dump(str(tmp_path), f, tiles=(2, 1, 1))
    g = fluid.Fluid((4, 3, 2), 5)
    restart.load(str(tmp_path), g)
    for n in restart.IO_FIELDS:
        assert np.array_equal(g[n], f[n]), n


@needs_lib
def test_many_datasets_span_several_symbol_table_nodes(tmp_path):
    f = random_fluid((3, 3, 3), seed=6, profiles=True)  # 10 datasets: two nodes of 8
    restart.dump(str(tmp_path), f, profiles=True)
    path = glob.glob(str(tmp_path / "*-*.hdf"))[0]
    t = h5read.File(path)
    assert len(t.datasets) == 10
    g = fluid.Fluid(f.shape, f.nspec)
    restart.load(str(tmp_path), g, profiles=True)
    for n in restart.IO_FIELDS + restart.PROFILE_FIELDS:
        assert np.array_equal(g[n], f[n]), n


# ---------------------------------------------------------------- errors

@needs_lib
def test_errors(tmp_path):
    lib = runtime.lib()
    f = random_fluid((4, 3, 2), seed=7)
    d = str(tmp_path / "r")
    parts = restart.dump(d, f)
    r = parts[0]
    v = f.view()
    H = abi.HTR_RESTART_HOST_VIEW
    g = fluid.Fluid(f.shape, f.nspec)
    gv = g.view()
    # missing directory or tile file
    assert lib.htr_restart_read_tile(b"/nonexistent", C.byref(gv), r, 5, H, None) == abi.HTR_ERR_IO
    assert lib.htr_restart_read_tile(d.encode(), C.byref(gv), abi.rect((0, 0, 0), (1, 1, 1)), 5, H,
                                     None) == abi.HTR_ERR_IO
    assert b"cannot open" in lib.htr_last_error()
    # profile fields asked for but not in the file
    g2 = random_fluid(f.shape, profiles=True)
    assert lib.htr_restart_read_tile(d.encode(), C.byref(g2.view()), r, 5, H | abi.HTR_RESTART_PROFILES,
                                     None) == abi.HTR_ERR_FORMAT
    assert b"MolarFracs_profile" in lib.htr_last_error()
    # another number of species
    g3 = fluid.Fluid(f.shape, 3)
    assert lib.htr_restart_read_tile(d.encode(), C.byref(g3.view()), r, 3, H, None) == abi.HTR_ERR_FORMAT
    # a file under another tile's name has the wrong shape
    other = abi.rect((0, 0, 0), (1, 2, 1))
    shutil.copy(restart.tile_filename(d, r), restart.tile_filename(d, other))
    assert lib.htr_restart_read_tile(d.encode(), C.byref(gv), other, 5, H, None) == abi.HTR_ERR_FORMAT
    # arguments
    nul = abi.htr_fluid_view()
    assert lib.htr_restart_write_tile(d.encode(), C.byref(nul), r, 5, H, None) == abi.HTR_ERR_ARGUMENT
    bad = f.view()
    bad.rho.stride[0] = 12
    assert lib.htr_restart_write_tile(d.encode(), C.byref(bad), r, 5, H, None) == abi.HTR_ERR_LAYOUT
    assert lib.htr_restart_write_tile(d.encode(), C.byref(v), abi.rect((2, 0, 0), (1, 2, 1)), 5, H,
                                      None) == abi.HTR_ERR_ARGUMENT
    assert lib.htr_restart_write_tile(None, C.byref(v), r, 5, H, None) == abi.HTR_ERR_ARGUMENT
    assert lib.htr_restart_write_tile(str(tmp_path / "no" / "dir").encode(), C.byref(v), r, 5, H,
                                      None) == abi.HTR_ERR_IO
    info = abi.htr_restart_info(1 << 40, 0.0, 0.0)
    t = (C.c_int64 * 3)(1, 1, 1)
    arr = (abi.htr_rect3 * 1)(r)
    assert lib.htr_restart_write_master(d.encode(), C.byref(info), r, t, arr, 5, None, None) == \
        abi.HTR_ERR_ARGUMENT
    # the state is rebuilt on device grids only
    with pytest.raises(abi.HtrError, match="device grid"):
        restart.load(d, fluid.Fluid(f.shape, f.nspec), mixture=C.c_void_p(1))
    # a grid of another size refuses the restart
    with pytest.raises(abi.HtrError, match="baseIndexSpace"):
        restart.load(d, fluid.Fluid((5, 3, 2), 5))
    # nothing was changed by the failed calls
    assert not g["rho"].any()


@needs_lib
def test_master_files_with_bad_sizes_or_tiles_are_rejected(tmp_path):
    """Attribute dimensions whose byte count overflows 64 bits, partitions
    reaching outside baseIndexSpace, and tilings that overlap or leave grid
    points uncovered are refused (HTR_ERR_FORMAT / HtrError), never read."""
    import struct

    from tests import h5_v2
    lib = runtime.lib()
    info, b, t = abi.htr_restart_info(), abi.htr_rect3(), (C.c_int64 * 3)()
    for name, dtype, dims in (("simTime", h5_v2.F64, [2 ** 61]), ("timeStep", h5_v2.int_type(8), [2 ** 32, 2 ** 32]),
                              ("timeStep", h5_v2.int_type(8), [2 ** 62, 3])):
        d = tmp_path / f"ov_{name}_{len(dims)}_{dims[0]}"
        d.mkdir()
        w = h5_v2.Writer()
        w.attribute("timeStep", h5_v2.int_type(8), [1], struct.pack("<q", 1))
        w.attribute("simTime", h5_v2.F64, [1], struct.pack("<d", 0.5))
        w.root_msgs = [m for m in w.root_msgs if name.encode() + b"\0" not in m[1]]
        w.attribute(name, dtype, dims, bytes(8))
        w.write(str(d / "master.hdf"))
        assert lib.htr_restart_read_master(str(d).encode(), C.byref(info), C.byref(b), t, None, 0) == \
            abi.HTR_ERR_FORMAT, name
    f = random_fluid((4, 3, 2), seed=9)
    d = str(tmp_path / "tiles")
    restart.dump(d, f, tiles=(2, 1, 1))
    master = os.path.join(d, "master.hdf")
    good = open(master, "rb").read()
    second = struct.pack("<6q", 2, 0, 0, 3, 2, 1)
    assert good.count(second) == 1
    with open(master, "wb") as fh:
        fh.write(good.replace(second, struct.pack("<6q", 2, 0, 0, 7, 2, 1)))
    parts = (abi.htr_rect3 * 2)()
    assert lib.htr_restart_read_master(d.encode(), C.byref(info), C.byref(b), t, parts, 2) == abi.HTR_ERR_FORMAT
    assert b"outside baseIndexSpace" in lib.htr_last_error()
    # the writer refuses such a partition too
    bounds = abi.rect((0, 0, 0), (3, 2, 1))
    out = (abi.htr_rect3 * 2)(abi.rect((0, 0, 0), (1, 2, 1)), abi.rect((2, 0, 0), (7, 2, 1)))
    t2 = (C.c_int64 * 3)(2, 1, 1)
    assert lib.htr_restart_write_master(d.encode(), C.byref(info), bounds, t2, out, 5, None, None) == \
        abi.HTR_ERR_ARGUMENT
    # tilings inside the grid that overlap or miss points
    for rects, msg in (((abi.rect((0, 0, 0), (2, 2, 1)), abi.rect((2, 0, 0), (3, 2, 1))), "overlap"),
                       ((abi.rect((0, 0, 0), (0, 2, 1)), abi.rect((2, 0, 0), (3, 2, 1))), "uncovered")):
        arr = (abi.htr_rect3 * 2)(*rects)
        abi.check(lib, lib.htr_restart_write_master(d.encode(), C.byref(info), bounds, t2, arr, 5, None, None))
        with pytest.raises(abi.HtrError, match=msg):
            restart.load(d, fluid.Fluid(f.shape, f.nspec))


@needs_lib
def test_corrupt_files_are_rejected_not_crashed(tmp_path):
    lib = runtime.lib()
    f = random_fluid((4, 3, 2), seed=8)
    d = str(tmp_path / "r")
    r = restart.dump(d, f)[0]
    path = restart.tile_filename(d, r)
    good = open(path, "rb").read()
    g = fluid.Fluid(f.shape, f.nspec)
    gv = g.view()
    H = abi.HTR_RESTART_HOST_VIEW

    def status(data):
        with open(path, "wb") as fh:
            fh.write(data)
        return lib.htr_restart_read_tile(d.encode(), C.byref(gv), r, 5, H, None)

    assert status(b"not an hdf5 file" * 64) == abi.HTR_ERR_FORMAT
    assert status(b"") == abi.HTR_ERR_FORMAT
    for cut in (8, 60, 100, 500, len(good) // 2, len(good) - 8):
        assert status(good[:cut]) == abi.HTR_ERR_FORMAT, cut
    # chunked storage is outside the subset: patch rho's layout class
    with open(path, "wb") as fh:
        fh.write(good)
    o = h5read.File(path)
    lay = [b for ty, _fl, b in o.messages["rho"] if ty == 0x08][0]
    at = good.index(lay)
    patched = bytearray(good)
    patched[at + 1] = 2
    assert status(bytes(patched)) == abi.HTR_ERR_UNSUPPORTED
    assert b"chunked" in lib.htr_last_error()
    # random byte flips in the metadata: any status, never a crash
    rng = np.random.default_rng(0)
    meta_end = min(len(good), 2048)
    seen = set()
    for _ in range(300):
        b = bytearray(good)
        for k in rng.integers(0, meta_end, size=3):
            b[k] ^= int(rng.integers(1, 256))
        seen.add(status(bytes(b)))
    assert seen <= {abi.HTR_OK, abi.HTR_ERR_FORMAT, abi.HTR_ERR_UNSUPPORTED, abi.HTR_ERR_IO, abi.HTR_ERR_ARGUMENT}
    assert status(good) == abi.HTR_OK


# ---------------------------------------------------------------- GPU

@pytest.mark.gpu
def test_restart_round_trip_device(tmp_path):
    """Device fields through the gather kernel, pinned staging and the file;
    128^3 points with five species make two slabs of MolarFracs."""
    import torch
    host = random_fluid((128, 128, 128), seed=9)
    dev = host.to_device("cuda:0")
    parts = restart.dump(str(tmp_path), dev, tiles=(1, 2, 1), time_step=7, sim_time=1.5)
    torch.cuda.synchronize()
    for r in parts:
        t = h5read.File(restart.tile_filename(str(tmp_path), r))
        for n in restart.IO_FIELDS:
            assert np.array_equal(t.datasets[n][0], tile_slice(host[n], r)), n
    back = fluid.Fluid(host.shape, host.nspec, device="cuda:0")
    info = restart.load(str(tmp_path), back)
    assert info["timeStep"] == 7 and info["simTime"] == 1.5
    out = back.to_host()
    for n in restart.IO_FIELDS:
        assert np.array_equal(out[n], host[n]), n


@pytest.mark.gpu
def test_run_continues_from_a_restart(tmp_path):
    """Step, dump, load into a fresh grid (conserved variables and properties
    rebuilt from the primitives, as a restarted run initialises them), then
    step both: the continued run agrees with the uninterrupted one within
    the RHS tolerance."""
    import torch

    import oracle
    from htr_gb300 import workloads
    from tests import util

    port = oracle.port_lib()
    host = workloads.taylor_green(32, seed=0)
    m = workloads.make_mixture_struct(port, host.meta["eos"], host.meta["mix"])
    workloads.derive_state(port, host, oracle.load_mixture(port, host.meta["eos"], m))
    gh = runtime.load_mixture(host.meta["eos"], m)
    a = host.to_device("cuda:0")
    dt = runtime.rk3_step(a, gh, scheme="Hybrid", cfl=0.8, chemistry=False)
    restart.dump(str(tmp_path), a, tiles=(2, 2, 2), time_step=1, sim_time=dt)
    b = host.to_device("cuda:0")  # grid fields (metrics, node types) of the same grid
    for n in restart.IO_FIELDS:
        b.arrays[n].zero_()
    info = restart.load(str(tmp_path), b, mixture=gh)
    assert info["timeStep"] == 1 and info["simTime"] == dt
    runtime.rk3_step(a, gh, scheme="Hybrid", dt=dt, chemistry=False)
    runtime.rk3_step(b, gh, scheme="Hybrid", dt=dt, chemistry=False)
    torch.cuda.synchronize()
    oa, ob = a.to_host(), b.to_host()
    util.check_fields(ob, oa, ("Conserved", "temperature", "pressure", "velocity", "rho"))


# ---------------------------------------------------------------- newer file format

def test_lookup3_published_vectors():
    """Bob Jenkins' lookup3.c self-test values for hashlittle."""
    from tests import h5_v2
    assert h5_v2.lookup3(b"", 0) == 0xDEADBEEF
    assert h5_v2.lookup3(b"", 0xDEADBEEF) == 0xBD5B7DDE
    assert h5_v2.lookup3(b"Four score and seven years ago", 0) == 0x17770551
    assert h5_v2.lookup3(b"Four score and seven years ago", 1) == 0xCD628161


@needs_lib
@pytest.mark.parametrize("kw", [{}, {"crt_order": True, "times": True}, {"split": True},
                                {"split": True, "crt_order": True}])
def test_reader_takes_the_newer_file_format(tmp_path, kw):
    """Superblock 2, version-2 object headers (checksummed; continuation
    blocks, creation order, times), link-message groups, attribute
    version 3: a tile file in that format loads like one in the earliest."""
    from tests import h5_v2
    lib = runtime.lib()
    f = random_fluid((5, 4, 3), seed=11)
    r = abi.rect((0, 0, 0), (4, 3, 2))
    d = tmp_path / "r"
    d.mkdir()
    path = restart.tile_filename(str(d), r)
    h5_v2.tile_file(path, f, r, restart.IO_FIELDS, **kw).write(path)
    g = fluid.Fluid(f.shape, f.nspec)
    gv = g.view()
    st = lib.htr_restart_read_tile(str(d).encode(), C.byref(gv), r, 5, abi.HTR_RESTART_HOST_VIEW, None)
    assert st == abi.HTR_OK, lib.htr_last_error()
    for n in restart.IO_FIELDS:
        assert np.array_equal(g[n], f[n]), n
    s = C.create_string_buffer(16)
    abi.check(lib, lib.htr_h5_string_attribute(path.encode(), None, b"note", 0, s, 16))
    assert s.value == b"latest"
    rank, dims, per = C.c_int(), (C.c_int64 * 8)(), C.c_int64()
    abi.check(lib, lib.htr_h5_dataset_shape(path.encode(), b"velocity", C.byref(rank), dims, C.byref(per)))
    assert (rank.value, list(dims[:3]), per.value) == (3, [3, 4, 5], 3)


@needs_lib
def test_newer_format_checksums_and_dense_groups(tmp_path):
    from tests import h5_v2
    lib = runtime.lib()
    f = random_fluid((4, 3, 2), seed=12)
    r = abi.rect((0, 0, 0), (3, 2, 1))
    path = restart.tile_filename(str(tmp_path), r)
    w = h5_v2.tile_file(path, f, r, restart.IO_FIELDS, split=True)
    w.write(path)
    good = open(path, "rb").read()
    g = fluid.Fluid(f.shape, f.nspec)
    gv = g.view()
    H = abi.HTR_RESTART_HOST_VIEW

    def status(data):
        with open(path, "wb") as fh:
            fh.write(data)
        return lib.htr_restart_read_tile(str(tmp_path).encode(), C.byref(gv), r, 5, H, None)

    # one flipped bit in each kind of metadata block: the superblock's base
    # address, an object header's chunk size, a continuation block's message
    for marker, off in ((b"\x89HDF", 12), (b"OHDR", 6), (b"OCHK", 6)):
        at = good.index(marker) + off
        bad = bytearray(good)
        bad[at] ^= 0x10
        assert status(bytes(bad)) == abi.HTR_ERR_FORMAT, marker
        assert b"checksum mismatch" in lib.htr_last_error(), (marker, lib.htr_last_error())
    assert status(good) == abi.HTR_OK
    # a link info message pointing at no fractal heap
    w.write(path, root_links_dense=True)
    assert lib.htr_restart_read_tile(str(tmp_path).encode(), C.byref(gv), r, 5, H, None) == abi.HTR_ERR_FORMAT
    assert b"FRHP" in lib.htr_last_error()


@needs_lib
@pytest.mark.parametrize("kw", [{}, {"crt_order": True, "split": True}])
def test_reader_takes_dense_groups(tmp_path, kw):
    """A tile with the three profile fields has ten links, more than the
    newer format keeps in the object header: they sit in a fractal heap
    indexed by a version-2 B-tree of name hashes."""
    from tests import h5_v2
    lib = runtime.lib()
    f = random_fluid((5, 4, 3), seed=13, profiles=True)
    r = abi.rect((0, 0, 0), (4, 3, 2))
    path = restart.tile_filename(str(tmp_path), r)
    names = restart.IO_FIELDS + restart.PROFILE_FIELDS
    h5_v2.tile_file(path, f, r, names, **kw).write(path, dense=True)
    assert b"FRHP" in open(path, "rb").read() and b"BTLF" in open(path, "rb").read()
    g = fluid.Fluid(f.shape, f.nspec)
    gv = g.view()
    st = lib.htr_restart_read_tile(str(tmp_path).encode(), C.byref(gv), r, 5,
                                   abi.HTR_RESTART_HOST_VIEW | abi.HTR_RESTART_PROFILES, None)
    assert st == abi.HTR_OK, lib.htr_last_error()
    for n in names:
        assert np.array_equal(g[n], f[n]), n
    # a flipped bit in the heap header or the name index is caught
    good = open(path, "rb").read()
    for marker in (b"FRHP", b"BTHD", b"BTLF"):
        bad = bytearray(good)
        bad[good.index(marker) + 8] ^= 0x04
        with open(path, "wb") as fh:
            fh.write(bytes(bad))
        assert lib.htr_restart_read_tile(str(tmp_path).encode(), C.byref(gv), r, 5,
                                         abi.HTR_RESTART_HOST_VIEW | abi.HTR_RESTART_PROFILES,
                                         None) == abi.HTR_ERR_FORMAT, marker
        assert b"checksum mismatch" in lib.htr_last_error(), marker
    # a name index deeper than one leaf is outside the subset (checksum kept valid)
    at = good.index(b"BTHD")
    bad = bytearray(good)
    bad[at + 12] = 1
    bad[at + 34:at + 38] = h5_v2.lookup3(bytes(bad[at:at + 34])).to_bytes(4, "little")
    with open(path, "wb") as fh:
        fh.write(bytes(bad))
    assert lib.htr_restart_read_tile(str(tmp_path).encode(), C.byref(gv), r, 5,
                                     abi.HTR_RESTART_HOST_VIEW | abi.HTR_RESTART_PROFILES,
                                     None) == abi.HTR_ERR_UNSUPPORTED
    assert b"deeper" in lib.htr_last_error()


@needs_lib
def test_reader_takes_dense_attributes(tmp_path):
    """Root attributes in dense storage (attribute info message, fractal
    heap, version-2 B-tree of type-8 records), links dense as well."""
    from tests import h5_v2
    lib = runtime.lib()
    f = random_fluid((4, 3, 2), seed=14, profiles=True)
    r = abi.rect((0, 0, 0), (3, 2, 1))
    path = restart.tile_filename(str(tmp_path), r)
    names = restart.IO_FIELDS + restart.PROFILE_FIELDS
    w = h5_v2.tile_file(path, f, r, names, crt_order=True)
    for k in range(9):
        w.attribute(f"extra{k}", h5_v2.string_type(8), [], f"value{k}".encode().ljust(8, b"\0"))
    w.write(path, dense=True, dense_attrs=True)
    s = C.create_string_buffer(16)
    for k in range(9):
        abi.check(lib, lib.htr_h5_string_attribute(path.encode(), None, f"extra{k}".encode(), 0, s, 16))
        assert s.value == f"value{k}".encode()
    abi.check(lib, lib.htr_h5_string_attribute(path.encode(), None, b"note", 0, s, 16))
    assert s.value == b"latest"
    g = fluid.Fluid(f.shape, f.nspec)
    gv = g.view()
    st = lib.htr_restart_read_tile(str(tmp_path).encode(), C.byref(gv), r, 5,
                                   abi.HTR_RESTART_HOST_VIEW | abi.HTR_RESTART_PROFILES, None)
    assert st == abi.HTR_OK, lib.htr_last_error()
    for n in names:
        assert np.array_equal(g[n], f[n]), n


# ---------------------------------------------------------------- golden files

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _golden_maker():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_restart_golden",
                                                  os.path.join(GOLDEN, "make_restart_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_oracle_reads_the_golden_restart():
    """The committed restart (tests/golden/restart) holds the seeded fields
    and the master attributes, read by the oracle alone."""
    mk = _golden_maker()
    f = mk.fields()
    d = os.path.join(GOLDEN, "restart")
    m = h5read.File(os.path.join(d, "master.hdf"))
    assert int(m.attrs["timeStep"]) == 1234 and float(m.attrs["simTime"]) == 0.5
    assert list(m.attrs["SpeciesNames"]) == [s.encode() for s in mk.SPECIES]
    parts, _ = m.datasets["partitions"]
    assert parts.shape == (1, 1, 2)
    for p in parts.ravel():
        lo, hi = p["lo"], p["hi"]
        name = f"{lo[0]},{lo[1]},{lo[2]}-{hi[0]},{hi[1]},{hi[2]}.hdf"
        t = h5read.File(os.path.join(d, name))
        for n in restart.IO_FIELDS:
            want = f[n][lo[2]:hi[2] + 1, lo[1]:hi[1] + 1, lo[0]:hi[0] + 1]
            assert np.array_equal(t.datasets[n][0], want), (name, n)


@needs_lib
def test_writer_reproduces_the_golden_restart(tmp_path):
    """The writer's bytes are stable: rewriting the golden restart gives the
    committed files byte for byte (no time stamps or addresses that vary)."""
    mk = _golden_maker()
    out = str(tmp_path / "r")
    mk.write(out)
    d = os.path.join(GOLDEN, "restart")
    assert sorted(os.listdir(out)) == sorted(os.listdir(d))
    for name in os.listdir(d):
        with open(os.path.join(d, name), "rb") as a, open(os.path.join(out, name), "rb") as b:
            assert a.read() == b.read(), name
