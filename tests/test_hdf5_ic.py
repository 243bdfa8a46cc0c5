"""Gadget-2 initial conditions read from HDF5 without libhdf5 (CPU only).

The reference's galaxy-collision example reads
examples/galaxy_collision/galaxy_collision_IC.hdf5 through libhdf5
(examples/galaxy_collision/c/galaxy_collision.c:109-293).  load_gadget2_ic
parses the file itself; these tests read that file where the reference is
present, and check that damaged or foreign files give errors, never a crash.

The values are pinned two ways: known entries of the file (first and last
particles of each species, the two masses, the unit attributes), and a
second read path that does not walk the HDF5 structures at all -- each array
the parser returns, written back as the little-endian FP32 the file stores,
must occur verbatim as one contiguous block of the file's bytes, and so must
the header attribute NumPart_ThisFile = (0, 40000, 20000, 0, 0, 0) as
uint32 (the counts the example reads, galaxy_collision.c:146-160).
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
    # known entries (the file stores FP32; every value is exactly an FP32)
    f32 = np.float32
    assert np.array_equal(x[0], f32([-94.13385009765625, -10.240921974182129, -7.942867279052734]))
    assert np.array_equal(v[0], f32([8.424066543579102, -51.35950469970703, -13.023665428161621]))
    assert np.array_equal(x[39999], f32([85.55107116699219, 36.82402038574219, -0.637717604637146]))
    assert np.array_equal(x[40000],
                          f32([-90.04521179199219, -33.32984161376953, -0.02418774925172329]))
    assert np.array_equal(v[40000], f32([45.37849044799805, 165.9688720703125, 50.6060791015625]))
    assert np.array_equal(x[-1], f32([92.15531921386719, 41.02614974975586, 6.769761085510254]))
    assert np.array_equal(v[-1], f32([-84.47198486328125, -73.0508041381836, 92.56161499023438]))
    assert m[0] == f32(0.0010463387006893754) and m[-1] == f32(0.00023251971288118511)


@pytest.mark.skipif(not IC.exists(), reason="reference initial conditions not present")
def test_values_occur_verbatim_in_the_file(lib, g):
    x, v, m, units = g.load_gadget2_ic(lib, IC)
    data = IC.read_bytes()
    blocks = [m[:40000], x[:40000], v[:40000], m[40000:], x[40000:], v[40000:]]
    offsets = []
    for arr in blocks:
        f32 = np.ascontiguousarray(arr, dtype="<f4")
        assert np.array_equal(f32.astype(np.float64), arr)     # exact FP32 values
        raw = f32.tobytes()
        off = data.find(raw[:64])
        assert off >= 0 and data[off:off + len(raw)] == raw
        offsets.append(off)
    assert len(set(offsets)) == len(offsets)                    # six distinct datasets
    assert data.find(np.array([0, 40000, 20000, 0, 0, 0], "<u4").tobytes()) >= 0
    for u in units:
        assert data.find(np.array([u], "<f8").tobytes()) >= 0


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
