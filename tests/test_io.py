"""Particle-field files (vpm_gb300.io, vpm_gb300.h5): the reference's save / read!
(src/FLOWVPM_utils.jl:148-371, 494-571), the .h5 and .xmf files it writes, and the HDF5 subset
those use. CPU only."""
import os
import xml.etree.ElementTree as ET

import numpy as np
import pytest

import vpm_gb300 as vpm
from vpm_gb300 import io as vio
from vpm_gb300.particlefield import C_INDEX, J_INDEX, STATIC_INDEX, U_INDEX, VORTICITY_INDEX


def _field(n, les=False, seed=0):
    rng = np.random.default_rng(seed)
    kw = {"SFS": vpm.SFS_Cd_twolevel_nobackscatter} if les else {}
    pf = vpm.ParticleField(n + 5, nt=17, t=0.085, **kw)
    pf.add_particles(rng.normal(size=(n, 3)), rng.normal(size=(n, 3)), rng.uniform(0.01, 0.1, n),
                     vol=rng.uniform(1e-4, 1e-3, n), circulation=rng.uniform(0.5, 2.0, n),
                     static=rng.uniform(size=n) < 0.2)
    P = pf.particles
    P[U_INDEX, :n] = rng.normal(size=(3, n))
    P[J_INDEX, :n] = rng.normal(size=(9, n))
    P[VORTICITY_INDEX, :n] = rng.normal(size=(3, n))
    P[C_INDEX, :n] = rng.normal(size=(3, n))
    return pf


@pytest.mark.parametrize("les", [False, True])
def test_save_read_round_trip(tmp_path, les):
    pf = _field(257, les=les)
    out = vio.save(pf, "field", path=str(tmp_path))
    assert out == "field.17.xmf;"
    assert os.path.exists(tmp_path / "field.17.xmf") and os.path.exists(tmp_path / "field.17.h5")
    back = vpm.ParticleField(300)
    vio.read(back, "field.17", path=str(tmp_path))
    n = pf.np
    assert back.np == n and back.nt == 17 and back.t == 0.085
    rows = [slice(0, 3), slice(3, 6), 6, 7, 8, STATIC_INDEX]      # what read! loads (utils.jl:541-560)
    for r in rows:
        np.testing.assert_array_equal(back.particles[r, :n], pf.particles[r, :n])
    np.testing.assert_array_equal(back.particles[C_INDEX, :n], pf.particles[C_INDEX, :n] if les else 0.0)


def test_xdmf_follows_the_reference_layout(tmp_path):
    pf = _field(40, les=True)
    vio.save(pf, "f", path=str(tmp_path), num=3)
    root = ET.parse(tmp_path / "f.3.xmf").getroot()
    assert root.tag == "Xdmf" and root.get("Version") == "3.0"
    grid = root.find("Domain/Grid")
    assert grid.get("Name") == "particles" and grid.get("GridType") == "Uniform"
    assert float(grid.find("Time").get("Value")) == 0.085
    assert grid.find("Geometry").get("Type") == "XYZ"
    assert grid.find("Geometry/DataItem").get("Dimensions") == "40 3"
    topo = grid.find("Topology")
    assert topo.get("Type") == "Polyvertex" and topo.get("Dimensions") == "40"
    names = [(a.get("Name"), a.get("Type")) for a in grid.findall("Attribute")]
    # the reference's attributes, in its order (src/FLOWVPM_utils.jl:277-356)
    assert names == [("Gamma", "Vector"), ("velocity", "Vector"), ("velocity gradient x", "Vector"),
                     ("velocity gradient y", "Vector"), ("velocity gradient z", "Vector"),
                     ("vorticity", "Vector"), ("sigma", "Scalar"), ("circulation", "Scalar"),
                     ("vol", "Scalar"), ("static", "Scalar"), ("C", "Vector")]
    datasets = {"Gamma": "Gamma", "velocity gradient x": "velocity_gradient_x", "velocity": "velocity",
                "velocity gradient y": "velocity_gradient_y", "velocity gradient z": "velocity_gradient_z"}
    assert grid.find("Geometry/DataItem").text == "f.3.h5:X"
    for a in grid.findall("Attribute"):
        item = a.find("DataItem")
        assert item.get("Format") == "HDF" and item.get("Precision") == "8"
        assert item.get("DataType") == ("Int" if a.get("Name") == "static" else "Float")
        assert item.text == "f.3.h5:" + datasets.get(a.get("Name"), a.get("Name"))
    # every item names a dataset of the .h5 file with the shape the item declares
    data = vio._datasets(str(tmp_path / "f.3.xmf"))
    assert len(data) == 12


def test_h5_datasets_as_the_reference_writes_them(tmp_path):
    """The .h5 holds the datasets of src/FLOWVPM_utils.jl:179-221 with HDF5.jl's types and
    shapes: np and nt int64 scalars, t a float64 scalar, the fields float64 (np x 3 or np)."""
    pf = _field(33)
    vio.save(pf, "g", path=str(tmp_path), add_num=False)
    from vpm_gb300 import h5
    names = h5.keys(str(tmp_path / "g.h5"))
    assert sorted(names) == sorted(["np", "nt", "t", "X", "Gamma", "sigma", "circulation", "vol", "static",
                                    "velocity", "velocity_gradient_x", "velocity_gradient_y",
                                    "velocity_gradient_z", "vorticity"])          # no C without SFS
    d = h5.read(str(tmp_path / "g.h5"))
    n = pf.np
    assert d["np"].shape == () and d["np"].dtype == np.int64 and d["np"] == n
    assert d["nt"].dtype == np.int64 and d["nt"] == 17
    assert d["t"].shape == () and d["t"].dtype == np.float64 and d["t"] == 0.085
    P = pf.particles
    np.testing.assert_array_equal(d["X"], P[0:3, :n].T)
    np.testing.assert_array_equal(d["velocity_gradient_y"], P[J_INDEX.start + 3:J_INDEX.start + 6, :n].T)
    np.testing.assert_array_equal(d["vorticity"], P[VORTICITY_INDEX, :n].T)
    assert d["static"].dtype == np.float64
    np.testing.assert_array_equal(d["static"], P[STATIC_INDEX, :n])


def test_h5_reader_reads_a_libhdf5_file():
    """The reader against a file libhdf5 wrote: scipy's MATLAB 7.3 test file (HDF5 after a
    512-byte user block) holds `testdouble` = pi/4 * (0..8), the value scipy's own MATLAB tests
    expect of it."""
    import scipy.io.matlab
    from vpm_gb300 import h5
    f = os.path.join(os.path.dirname(scipy.io.matlab.__file__), "tests", "data", "testhdf5_7.4_GLNX86.mat")
    if not os.path.exists(f):
        pytest.skip("scipy's HDF5 test file is not installed")
    d = h5.read(f)
    assert list(d) == ["testdouble"] and d["testdouble"].shape == (9, 1)
    np.testing.assert_array_equal(d["testdouble"].ravel(), np.pi / 4 * np.arange(9.0))


def test_h5_encodings_match_libhdf5(tmp_path):
    """The float64 datatype and fill-value messages written here are byte for byte the ones
    libhdf5 wrote for a float64 dataset (scipy's MATLAB 7.3 test file)."""
    import scipy.io.matlab
    from vpm_gb300 import h5
    f = os.path.join(os.path.dirname(scipy.io.matlab.__file__), "tests", "data", "testhdf5_7.4_GLNX86.mat")
    if not os.path.exists(f):
        pytest.skip("scipy's HDF5 test file is not installed")
    ref = h5._File(open(f, "rb").read())
    ref_msgs = dict(ref.messages(ref.group(ref.root_ohdr, ref.root_cache)["testdouble"]))
    h5.write(str(tmp_path / "x.h5"), {"a": np.zeros(3)})
    ours = h5._File(open(tmp_path / "x.h5", "rb").read())
    msgs = dict(ours.messages(ours.group(ours.root_ohdr, ours.root_cache)["a"]))
    assert msgs[h5.MSG_DATATYPE] == ref_msgs[h5.MSG_DATATYPE]
    assert msgs[h5.MSG_FILL] == ref_msgs[h5.MSG_FILL]


def test_h5_file_structure(tmp_path):
    """The invariants libhdf5 relies on when it opens a file: the superblock's end-of-file
    address is the file size, the heap's free list is empty, every symbol-table node holds at
    most 2 x 4 names in byte order, and B-tree key i+1 is the last name of child i."""
    from vpm_gb300 import h5
    rng = np.random.default_rng(1)
    names = [f"d{i:02d}" for i in range(19)] + ["np", "X", "velocity_gradient_x"]
    h5.write(str(tmp_path / "s.h5"), {k: rng.normal(size=(i + 1,)) for i, k in enumerate(names)})
    raw = (tmp_path / "s.h5").read_bytes()
    f = h5._File(raw)
    assert int.from_bytes(raw[40:48], "little") == len(raw)
    tree, heap = f.root_cache
    assert raw[heap:heap + 4] == b"HEAP" and int.from_bytes(raw[heap + 16:heap + 24], "little") == h5.HEAP_FREE_NULL
    hdata = int.from_bytes(raw[heap + 24:heap + 32], "little")
    name = lambda off: raw[hdata + off:raw.index(b"\0", hdata + off)]
    used = int.from_bytes(raw[tree + 6:tree + 8], "little")
    assert used == 3
    keys = [int.from_bytes(raw[tree + 24 + 16 * i:tree + 32 + 16 * i], "little") for i in range(used + 1)]
    kids = [int.from_bytes(raw[tree + 32 + 16 * i:tree + 40 + 16 * i], "little") for i in range(used)]
    assert name(keys[0]) == b""
    seen = []
    for i, k in enumerate(kids):
        assert raw[k:k + 4] == b"SNOD"
        ns = int.from_bytes(raw[k + 6:k + 8], "little")
        assert 1 <= ns <= 8
        child = [name(int.from_bytes(raw[k + 8 + 40 * e:k + 16 + 40 * e], "little")) for e in range(ns)]
        assert child == sorted(child) and name(keys[i + 1]) == child[-1]
        seen += child
    assert seen == sorted(n.encode() for n in names)
    assert sorted(h5.keys(str(tmp_path / "s.h5"))) == sorted(names)


def test_empty_field_saves_one_dummy_particle(tmp_path):
    pf = vpm.ParticleField(10, nt=4, t=0.5)
    vio.save(pf, "e", path=str(tmp_path))
    back = vio.read(vpm.ParticleField(2), "e.4.h5", path=str(tmp_path))
    assert back.np == 1 and back.nt == 4 and back.t == 0.5
    np.testing.assert_array_equal(back.particles[0:7, 0], 0.0)


def test_read_overflow_and_append(tmp_path):
    pf = _field(20)
    vio.save(pf, "h", path=str(tmp_path))
    with pytest.raises(RuntimeError, match="max number of particles"):
        vio.read(vpm.ParticleField(19), "h.17", path=str(tmp_path))
    two = vpm.ParticleField(40)
    vio.read(two, "h.17", path=str(tmp_path))
    vio.read(two, "h.17.h5", path=str(tmp_path), overwrite=False, load_time=False)
    assert two.np == 40
    np.testing.assert_array_equal(two.particles[0:9, 20:40], pf.particles[0:9, :20])


def test_run_vpm_saves_on_the_reference_cadence(tmp_path):
    """run_vpm with save_path (src/FLOWVPM_utils.jl:122-126): step 0, every nsteps_save steps and the
    last step are saved; the last file reads back as the final state.  The oracle is the UJ hook."""
    import oracle

    def uj_oracle(pfield, rbf=False, sfs=False, reset=True, reset_sfs=False, **kw):
        flags = (oracle.RESET if reset else 0) | (oracle.RESET_SFS if reset_sfs else 0) | \
                (oracle.SFS if sfs else 0) | (oracle.TRANSPOSED if pfield.transposed else 0)
        oracle.uj_direct(pfield.particles, pfield.np, pfield.kernel.kid, flags)

    rng = np.random.default_rng(3)
    pf = vpm.ParticleField(64, formulation=vpm.rVPM, kernel=vpm.gaussianerf, UJ=uj_oracle)
    pf.add_particles(rng.uniform(0, 1, (48, 3)), rng.normal(0, 1e-2, (48, 3)), np.full(48, 0.1))
    vpm.run_vpm(pf, 1e-3, 5, save_path=str(tmp_path / "run"), run_name="ring", nsteps_save=2)
    saved = sorted(f for f in os.listdir(tmp_path / "run") if f.endswith(".xmf"))
    assert saved == ["ring.0.xmf", "ring.2.xmf", "ring.4.xmf", "ring.5.xmf"]
    back = vio.read(vpm.ParticleField(64), "ring.5", path=str(tmp_path / "run"))
    assert back.nt == 5 and back.np == 48
    np.testing.assert_array_equal(back.particles[0:7, :48], pf.particles[0:7, :48])


def test_save_device_state(tmp_path):
    """The device-resident state (here on CPU tensors) goes to the same files."""
    import torch
    from vpm_gb300.device_step import DeviceField
    rng = np.random.default_rng(5)
    n = 30
    t = lambda a: torch.tensor(a, dtype=torch.float64)
    fld = DeviceField(t(rng.normal(size=(n, 3))), t(rng.normal(size=(n, 3))), t(rng.uniform(0.01, 0.1, n)),
                      nt=9, t=0.045)
    fld.J.copy_(t(rng.normal(size=(n, 9))))
    fld.C.copy_(t(rng.normal(size=(n, 3))))
    vio.save_device(fld, "dev", les=True, path=str(tmp_path))
    back = vio.read(vpm.ParticleField(n), "dev.9", path=str(tmp_path))
    assert back.np == n and back.nt == 9 and back.t == 0.045
    np.testing.assert_array_equal(back.particles[0:3, :n], fld.x.numpy().T)
    np.testing.assert_array_equal(back.particles[3:6, :n], fld.gam.numpy().T)
    np.testing.assert_array_equal(back.particles[6, :n], fld.sig.numpy())
    np.testing.assert_array_equal(back.particles[C_INDEX, :n], fld.C.numpy().T)
    data = vio._datasets(str(tmp_path / "dev.9.xmf"))
    np.testing.assert_array_equal(data["velocity_gradient_z"], fld.J.numpy()[:, 6:9])
