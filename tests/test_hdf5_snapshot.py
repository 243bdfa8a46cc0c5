"""HDF5 snapshots in grav_sim's layout, written without libhdf5 (CPU only).

grav_sim's output method 3 (src/output.c:483-695) writes, per snapshot,
group /Header with the int attributes NumFilesPerSnapshot, NumPart_ThisFile,
NumPart_Total and the double attribute Time, and group /PartType0 with the
datasets ParticleIDs (int32 [N]), Masses ([N]), Coordinates ([N][3]) and
Velocities ([N][3]), FP32 or FP64 by the output dtypes.  Its cosmological
snapshots (src/output.c:697-900) add Redshift, Omega0, OmegaLambda and a
/Units group, with scalar attributes.

No libhdf5 or h5py exists on these machines, so the files are read back two
independent ways: the library's own HDF5 reader (the one that reads the
reference's h5py-written galaxy_collision_IC.hdf5, test_hdf5_ic.py), and the
walker of h5walk.py, written from the published HDF5 file-format
specification.
"""
import numpy as np
import pytest

from h5walk import Walker
from oracle.reference import REF_DIR

IC = REF_DIR / "examples" / "galaxy_collision" / "galaxy_collision_IC.hdf5"


@pytest.mark.skipif(not IC.exists(), reason="reference initial conditions not present")
def test_walker_reads_the_reference_ic_file(lib, g):
    """The walker itself, pinned on a file written by h5py: it returns what the
    library's reader returns for the reference's galaxy-collision initial
    conditions, and the header and unit attributes that file holds."""
    x, v, m, units = g.load_gadget2_ic(lib, IC)
    w = Walker(IC)
    assert sorted(w.children(w.root)) == ["Header", "PartType1", "PartType2", "Units"]
    wx = np.concatenate([w.dataset(f"/PartType{k}/Coordinates") for k in (1, 2)])
    wv = np.concatenate([w.dataset(f"/PartType{k}/Velocities") for k in (1, 2)])
    wm = np.concatenate([w.dataset(f"/PartType{k}/Masses") for k in (1, 2)])
    assert np.array_equal(wx.astype(np.float64), x) and np.array_equal(wv.astype(np.float64), v)
    assert np.array_equal(wm.astype(np.float64), m)
    hdr = w.attributes("/Header")
    assert hdr["NumPart_ThisFile"][0].tolist() == [0, 40000, 20000, 0, 0, 0]
    u = {k: val.tolist() for k, (val, shape) in w.attributes("/Units").items()}
    assert (u["Unit length in cgs (U_L)"], u["Unit mass in cgs (U_M)"],
            u["Unit time in cgs (U_t)"]) == ([units[0]], [units[1]], [units[2]])


def _state(n, seed):
    rng = np.random.default_rng(seed)
    ids = rng.permutation(n).astype(np.int32)
    return (ids, rng.normal(size=(n, 3)), rng.normal(size=(n, 3)),
            rng.uniform(0.5, 2.0, n))


@pytest.mark.parametrize("n", [0, 1, 7, 1000])
@pytest.mark.parametrize("dtypes", [(2, 2, 2), (1, 1, 1), (1, 2, 1)])
def test_snapshot_round_trip(lib, g, tmp_path, n, dtypes):
    ids, x, v, m = _state(n, n + 10 * dtypes[0] + dtypes[1])
    t = 0.123456789012345678
    path = tmp_path / "snapshot_00003.hdf5"
    g.write_snapshot_hdf5(lib, path, ids, x, v, m, t, dtypes)
    as_out = {1: lambda a: a.astype(np.float32).astype(np.float64), 2: lambda a: a}
    want = {"Coordinates": as_out[dtypes[0]](x), "Velocities": as_out[dtypes[1]](v),
            "Masses": as_out[dtypes[2]](m), "ParticleIDs": ids.astype(np.float64)}
    # the walker
    w = Walker(path)
    assert sorted(w.children(w.root)) == ["Header", "PartType0"]
    assert sorted(w.children(w.lookup("/PartType0"))) == sorted(want)
    assert w.children(w.lookup("/Header")) == {}
    for name, arr in want.items():
        got = w.dataset(f"/PartType0/{name}")
        assert got.shape == arr.shape
        kind = {"Coordinates": 0, "Velocities": 1, "Masses": 2}.get(name)
        assert got.dtype == (np.dtype("<i4") if kind is None
                             else np.dtype("<f4" if dtypes[kind] == 1 else "<f8"))
        assert np.array_equal(got.astype(np.float64), arr), name
    attrs = w.attributes("/Header")
    assert sorted(attrs) == ["NumFilesPerSnapshot", "NumPart_ThisFile", "NumPart_Total", "Time"]
    assert attrs["NumFilesPerSnapshot"][0].tolist() == [1]
    assert attrs["NumPart_ThisFile"][0].tolist() == [n] and attrs["NumPart_Total"][0].tolist() == [n]
    assert attrs["Time"][0].dtype == np.dtype("<f8") and attrs["Time"][0].tolist() == [t]
    assert all(shape == (1,) for _, shape in attrs.values())
    # the library's reader
    for name, arr in want.items():
        got = g.hdf5_read(lib, path, f"/PartType0/{name}")
        assert np.array_equal(got, arr.reshape(-1)), name
    assert g.hdf5_read(lib, path, "/Header", "Time").tolist() == [t]
    assert g.hdf5_read(lib, path, "/Header", "NumPart_Total").tolist() == [float(n)]


def test_snapshot_is_deterministic(lib, g, tmp_path):
    ids, x, v, m = _state(64, 3)
    g.write_snapshot_hdf5(lib, tmp_path / "a.hdf5", ids, x, v, m, 1.5)
    g.write_snapshot_hdf5(lib, tmp_path / "b.hdf5", ids, x, v, m, 1.5)
    assert (tmp_path / "a.hdf5").read_bytes() == (tmp_path / "b.hdf5").read_bytes()


def test_snapshot_errors(lib, g, tmp_path):
    ids, x, v, m = _state(4, 4)
    with pytest.raises(g.GravError) as e:
        g.write_snapshot_hdf5(lib, tmp_path / "missing_dir" / "s.hdf5", ids, x, v, m, 0.0)
    assert e.value.code == 5      # GRAV_OS_ERROR
    path = tmp_path / "s.hdf5"
    g.write_snapshot_hdf5(lib, path, ids, x, v, m, 0.0)
    with pytest.raises(g.GravError):
        g.hdf5_read(lib, path, "/PartType1/Masses")
    with pytest.raises(g.GravError):
        g.hdf5_read(lib, path, "/Header", "Redshift")
    # a truncated file gives an error, never a crash
    data = path.read_bytes()
    for cut in (8, 96, len(data) // 2, len(data) - 8):
        bad = tmp_path / f"cut{cut}.hdf5"
        bad.write_bytes(data[:cut])
        with pytest.raises(g.GravError):
            g.hdf5_read(lib, bad, "/PartType0/Velocities")
