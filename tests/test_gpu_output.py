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

import pytest

from conftest import cases, golden

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
