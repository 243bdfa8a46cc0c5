"""CSV snapshots written during launch_simulation, byte for byte.

The golden files are the snapshots grav_sim itself wrote for the same runs
(src/output.c:340-470 called from the integrator loops: src/integrator.c
:326-415 and :1043-1071, src/integrator_rk_embedded.c:690-880,
src/integrator_ias15.c:380-520, src/integrator_whfast.c:249-364).  With the
FP64 reference-order forces every number printed with "%.17g" must agree,
as must the file numbering, the metadata lines and the snapshot times.

grav_sim's Python entry point leaves the status of the initial snapshot
uninitialised; this library writes t = 0 and the integrator's dt there, so
those two lines of snapshot_00000.csv are not compared when output_initial
is set.
"""
import json

import numpy as np
import pytest

from conftest import cases, golden
from h5walk import Walker

pytestmark = pytest.mark.gpu

CASES = cases(golden("output"))
# reference acceleration code -> the GPU code that reproduces it bit for bit
GPU_METHOD = {1: 111, 2: 102}


def _without_status_lines(text: bytes) -> bytes:
    lines = text.split(b"\n")
    assert lines[2].startswith(b"# time: ") and lines[3].startswith(b"# dt: ")
    return b"\n".join(lines[:2] + lines[4:])


@pytest.mark.parametrize("name", sorted(CASES))
def test_snapshots_match_reference_bytes(lib, g, tmp_path, name):
    c = dict(CASES[name])
    args = json.loads(bytes(c.pop("args.json")).decode())
    x, v, m, G = c.pop("x0").copy(), c.pop("v0").copy(), c.pop("m0").copy(), float(c.pop("G"))
    extra, oargs = args["extra"], args["output"]
    out_dir = tmp_path / "snaps"
    g.launch_simulation(lib, x, v, m, G, integrator=args["integrator"], dt=args["dt"],
                        tf=args["tf"], method=GPU_METHOD[args["method"]],
                        softening_length=extra.get("eps", 0.0),
                        tolerance=extra.get("tolerance", -1.0),
                        output_method=g.OUTPUT_METHOD_CSV, output_dir=str(out_dir) + "/", **oargs)
    files = sorted(p.name for p in out_dir.iterdir())
    assert files == sorted(c), (files, sorted(c))
    for f in files:
        got, want = (out_dir / f).read_bytes(), bytes(c[f])
        if f == "snapshot_00000.csv" and oargs["output_initial"]:
            got, want = _without_status_lines(got), _without_status_lines(want)
        assert got == want, f


def test_initial_snapshot_status_lines(lib, g, tmp_path):
    """Initial snapshot: t = 0 and the integrator's dt (leapfrog case)."""
    c = CASES["leapfrog"]
    args = json.loads(bytes(c["args.json"]).decode())
    out_dir = tmp_path / "snaps"
    g.launch_simulation(lib, c["x0"].copy(), c["v0"].copy(), c["m0"].copy(), float(c["G"]),
                        integrator=4, dt=args["dt"], tf=args["dt"], method=111,
                        softening_length=0.01, output_method=g.OUTPUT_METHOD_CSV,
                        output_dir=str(out_dir) + "/", output_initial=True, output_interval=1.0)
    lines = (out_dir / "snapshot_00000.csv").read_text().split("\n")
    assert lines[2] == "# time: 0" and lines[3] == f"# dt: {args['dt']!r}"
    assert sorted(p.name for p in out_dir.iterdir()) == ["snapshot_00000.csv"]


def _csv_values(text: bytes):
    """(time, ids, m, x, v) of one of the reference's CSV snapshots."""
    lines = text.decode().strip().split("\n")
    t = float(lines[2].split(": ")[1])
    rows = np.array([[float(f) for f in ln.split(",")] for ln in lines[5:]]).reshape(-1, 8)
    return t, rows[:, 0], rows[:, 1], rows[:, 2:5], rows[:, 5:8]


@pytest.mark.parametrize("name", sorted(CASES))
def test_hdf5_snapshots_hold_the_reference_csv_values(lib, g, tmp_path, name):
    """The same runs with output method 3: one snapshot_%05d.hdf5 per CSV file
    the reference wrote, holding the same numbers (exactly for FP64 output,
    to FP32 rounding for FP32 output) and the same time."""
    c = dict(CASES[name])
    args = json.loads(bytes(c.pop("args.json")).decode())
    x, v, m, G = c.pop("x0").copy(), c.pop("v0").copy(), c.pop("m0").copy(), float(c.pop("G"))
    extra, oargs = args["extra"], args["output"]
    out_dir = tmp_path / "snaps"
    g.launch_simulation(lib, x, v, m, G, integrator=args["integrator"], dt=args["dt"],
                        tf=args["tf"], method=GPU_METHOD[args["method"]],
                        softening_length=extra.get("eps", 0.0),
                        tolerance=extra.get("tolerance", -1.0),
                        output_method=g.OUTPUT_METHOD_HDF5, output_dir=str(out_dir) + "/", **oargs)
    files = sorted(p.name for p in out_dir.iterdir())
    assert files == sorted(f.replace(".csv", ".hdf5") for f in c)
    dtypes = {"Coordinates": oargs.get("coordinate_output_dtype", 2),
              "Velocities": oargs.get("velocity_output_dtype", 2),
              "Masses": oargs.get("mass_output_dtype", 2)}
    for f in sorted(c):
        t, ids, mm, xx, vv = _csv_values(bytes(c[f]))
        w = Walker(out_dir / f.replace(".csv", ".hdf5"))
        assert np.array_equal(w.dataset("/PartType0/ParticleIDs"), ids.astype(np.int32))
        for key, want in (("Masses", mm), ("Coordinates", xx), ("Velocities", vv)):
            got = w.dataset(f"/PartType0/{key}").astype(np.float64)
            assert got.shape == want.shape, key
            if dtypes[key] == 2:
                assert np.array_equal(got, want), (f, key)
            else:
                tol = np.abs(want) * 2.0 ** -23
                assert (np.abs(got - want) <= tol).all(), (f, key)
        hdr = w.attributes("/Header")
        assert hdr["NumPart_Total"][0].tolist() == [len(ids)]
        if not (f == "snapshot_00000.csv" and oargs["output_initial"]):
            assert hdr["Time"][0].tolist() == [t], f


def test_cosmological_hdf5_snapshots(lib, g, orc, tmp_path):
    """Cosmological snapshots (src/output.c:697-900) through
    launch_cosmological_simulation: the initial one holds the input state,
    one per step follows at an interval of one step, the last holds the
    returned x and v, v is momentum / a^2 as the oracle computes it, and the
    header carries Redshift = 1/a - 1, Omega0, OmegaLambda and /Units."""
    cs = cases(golden("pm"))["cosmo"]
    kw = json.loads(bytes(cs["args.json"]).decode())
    x, v = cs["x0"].copy(), cs["v0"].copy()
    units = (1.989e43, 3.085678e24, 3.085678e19)
    out_dir = tmp_path / "cosmo"
    st = g.launch_cosmological_simulation(lib, x, v, cs["m"], **kw,
                                          output_method=g.OUTPUT_METHOD_HDF5,
                                          output_dir=str(out_dir) + "/", output_initial=True,
                                          output_interval=kw["dt"] * (1 - 1e-9), units=units)
    steps = int(cs["steps"])
    assert st.num_steps == steps
    files = sorted(p.name for p in out_dir.iterdir())
    assert files == [f"snapshot_{k:05d}.hdf5" for k in range(steps + 1)]
    w0 = Walker(out_dir / files[0])
    assert np.array_equal(w0.dataset("/PartType0/Coordinates"), cs["x0"])
    assert np.array_equal(w0.dataset("/PartType0/Velocities"), cs["v0"])
    assert w0.attributes("/Header")["Time"][0].tolist() == [kw["a_begin"]]
    wl = Walker(out_dir / files[-1])
    assert np.array_equal(wl.dataset("/PartType0/Coordinates"), x)
    assert np.array_equal(wl.dataset("/PartType0/Velocities"), v)
    assert np.array_equal(wl.dataset("/PartType0/Masses"), cs["m"])
    assert np.abs(x - cs["x"]).max() <= 1e-9 * kw["box_width"]
    _, _, _, v_last = orc.leapfrog_cosmology(
        cs["x0"], cs["v0"], cs["m"], kw["h"], kw["omega_m"], kw["omega_lambda"],
        kw["box_center"], kw["box_width"], kw["dt"], kw["a_begin"], kw["a_final"],
        kw["pm_grid_size"], velocities=True)
    assert np.abs(v - v_last).max() <= 1e-9 * np.abs(v_last).max()
    hdr = {k: (val.tolist(), shape) for k, (val, shape) in wl.attributes("/Header").items()}
    a = float(st.t)
    assert hdr["Time"] == ([a], ()) and hdr["Redshift"] == ([1.0 / a - 1.0], ())
    assert hdr["Omega0"] == ([kw["omega_m"]], ()) and hdr["OmegaLambda"] == ([kw["omega_lambda"]], ())
    assert hdr["NumPart_ThisFile"] == ([cs["m"].size], (1,))
    u = {k: val.tolist() for k, (val, shape) in wl.attributes("/Units").items()}
    assert u == {"Unit current in cgs (U_I)": [1.0], "Unit length in cgs (U_L)": [units[1]],
                 "Unit mass in cgs (U_M)": [units[0]], "Unit time in cgs (U_t)": [units[2]],
                 "Unit temperature in cgs (U_T)": [1.0]}


def test_cosmological_csv_output_is_refused(lib, g, tmp_path):
    cs = cases(golden("pm"))["cosmo"]
    kw = json.loads(bytes(cs["args.json"]).decode())
    with pytest.raises(g.GravError):
        g.launch_cosmological_simulation(lib, cs["x0"].copy(), cs["v0"].copy(), cs["m"], **kw,
                                         output_method=g.OUTPUT_METHOD_CSV,
                                         output_dir=str(tmp_path) + "/")
