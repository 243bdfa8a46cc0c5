"""Gadget-2 initial conditions read from HDF5 without libhdf5 (CPU only).

The reference's galaxy-collision example reads
examples/galaxy_collision/galaxy_collision_IC.hdf5 through libhdf5
(examples/galaxy_collision/c/galaxy_collision.c:109-293).  load_gadget2_ic
parses the file itself; these tests read that file where the reference is
present, and check that damaged or foreign files give errors, never a crash.
"""

import numpy as np
import pytest

from oracle.reference import REF_DIR

IC = REF_DIR / "examples" / "galaxy_collision" / "galaxy_collision_IC.hdf5"


@pytest.mark.skipif(not IC.exists(), reason="reference initial conditions not present")
def test_reads_reference_galaxy_collision_ic(lib, g):
    x, v, m, units = g.load_gadget2_ic(lib, IC)
    assert x.shape == (60000, 3) and v.shape == (60000, 3) and m.shape == (60000,)
    # Units: kpc, 1e10 solar masses and kpc / (km/s), in cgs
    assert units == (3.085678e21, 1.989e43, 3.085678e16)
    assert np.isfinite(x).all() and np.isfinite(v).all() and (m > 0).all()
    # PartType1 (halo) first, then PartType2 (disk): two equal-mass species
    masses, counts = np.unique(m, return_counts=True)
    assert len(masses) == 2 and sorted(counts.tolist()) == [20000, 40000]
    assert (m[:40000] == m[0]).all() and (m[40000:] == m[-1]).all()
    # two galaxies on either side of the origin
    assert x[:, 0].min() < -50 and x[:, 0].max() > 50


@pytest.mark.skipif(not IC.exists(), reason="reference initial conditions not present")
def test_damaged_files_give_errors(lib, g, tmp_path):
    data = IC.read_bytes()
    for name, blob in [("truncated.hdf5", data[:5000]), ("header_only.hdf5", data[:96]),
                       ("zeros.hdf5", data[:8] + bytes(4096)),
                       ("flipped.hdf5", data[:700] + bytes(b ^ 0xFF for b in data[700:900])
                        + data[900:])]:
        f = tmp_path / name
        f.write_bytes(blob)
        with pytest.raises(g.GravError):
            g.load_gadget2_ic(lib, f)


def test_foreign_and_missing_files(lib, g, tmp_path):
    f = tmp_path / "not.hdf5"
    f.write_bytes(b"particle_id,m,x,y,z\n" * 10)
    with pytest.raises(g.GravError) as e:
        g.load_gadget2_ic(lib, f)
    assert "not an HDF5 file" in str(e.value)
    with pytest.raises(g.GravError) as e:
        g.load_gadget2_ic(lib, tmp_path / "absent.hdf5")
    assert "Failed to open" in str(e.value)
