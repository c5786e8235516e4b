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


def _crafted_h5(path):
    """A file that uses what the writer never writes but the reader reads: superblock version 1,
    a two-level group B-tree (an internal node over two leaf nodes), a compact dataset, a
    big-endian float64 and a big-endian int32 dataset, and a dataset whose object header continues
    in a second chunk (a continuation message). Returns the expected {name: array}."""
    import struct
    from vpm_gb300 import h5
    expect = {"a_compact": np.arange(5, dtype=np.float64) / 8,
              "b_be_f64": np.linspace(-1, 1, 6).reshape(2, 3),
              "c_be_i32": np.array([-7, 0, 9], dtype=np.int32),
              "d_cont": np.array([3.25, -1.5])}
    names = sorted(expect)
    heap_data, off = b"\0" * 8, {}
    for nm in names:
        off[nm] = len(heap_data)
        heap_data += nm.encode() + b"\0" * (h5._pad8(len(nm) + 1) - len(nm))
    be_f64 = struct.pack("<B3BI HHBBBBI", 0x11, 0x21, 63, 0, 8, 0, 64, 52, 11, 0, 52, 1023)   # byte order bit set
    be_i32 = struct.pack("<B3BI HH", 0x10, 0x09, 0, 0, 4, 0, 32)
    le_f64 = h5._datatype_msg(np.dtype(np.float64))
    sb, pos = 100, {}                      # superblock v1 is 100 bytes with 8-byte offsets
    layout = ["root", "heap", "inner", "leaf0", "leaf1", "snod0", "snod1"] + names + ["cont", "data"]
    sizes = {"root": 16 + 32, "heap": 32 + len(heap_data), "inner": h5._TREE_BYTES, "leaf0": h5._TREE_BYTES,
             "leaf1": h5._TREE_BYTES, "snod0": h5._SNOD_BYTES, "snod1": h5._SNOD_BYTES}
    data = {"b_be_f64": expect["b_be_f64"].astype(">f8").tobytes(), "c_be_i32": expect["c_be_i32"].astype(">i4").tobytes(),
            "d_cont": expect["d_cont"].astype("<f8").tobytes()}
    msgs = {}
    msgs["a_compact"] = [(h5.MSG_DATATYPE, 1, le_f64), (h5.MSG_DATASPACE, 0, h5._dataspace_msg((5,))),
                         (h5.MSG_LAYOUT, 1, struct.pack("<BBH", 3, 0, 40) + expect["a_compact"].tobytes())]
    p = sb
    for k in layout:
        pos[k] = p
        if k in names:
            if k == "b_be_f64":
                msgs[k] = [(h5.MSG_DATATYPE, 1, be_f64), (h5.MSG_DATASPACE, 0, h5._dataspace_msg((2, 3))),
                           (h5.MSG_LAYOUT, 1, b"\0" * 18)]
            elif k == "c_be_i32":
                msgs[k] = [(h5.MSG_DATATYPE, 1, be_i32), (h5.MSG_DATASPACE, 0, h5._dataspace_msg((3,))),
                           (h5.MSG_LAYOUT, 1, b"\0" * 18)]
            elif k == "d_cont":
                msgs[k] = [(h5.MSG_DATATYPE, 1, le_f64), (h5.MSG_CONTINUATION, 0, b"\0" * 16)]
            sizes[k] = len(h5._object_header(msgs[k]))
        elif k == "cont":
            sizes[k] = 8 + 16 + 8 + 24               # the dataspace and layout messages of d_cont
        elif k == "data":
            sizes[k] = sum(len(v) for v in data.values())
        p += sizes[k]
    eof = p
    dpos, q = {}, pos["data"]
    for k in ("b_be_f64", "c_be_i32", "d_cont"):
        dpos[k] = q
        q += len(data[k])
    for k in ("b_be_f64", "c_be_i32"):
        msgs[k][2] = (h5.MSG_LAYOUT, 1, struct.pack("<BBQQ", 3, 1, dpos[k], len(data[k])))
    msgs["d_cont"][1] = (h5.MSG_CONTINUATION, 0, struct.pack("<QQ", pos["cont"], sizes["cont"]))
    out = bytearray(eof)
    out[0:sb] = (h5.SIGNATURE + struct.pack("<8BHHI", 1, 0, 0, 0, 0, 8, 8, 0, 4, 16, 0) + struct.pack("<HH", 32, 0)
                 + struct.pack("<QQQQ", 0, h5.UNDEF, eof, h5.UNDEF) + struct.pack("<QQII", 0, pos["root"], 0, 0) + b"\0" * 16)
    root = h5._object_header([(h5.MSG_SYMTAB, 1, struct.pack("<QQ", pos["inner"], pos["heap"])), (h5.MSG_NIL, 0, b"")])
    out[pos["root"]:pos["root"] + len(root)] = root
    out[pos["heap"]:pos["heap"] + 32] = b"HEAP" + struct.pack("<B3xQQQ", 0, len(heap_data), 1, pos["heap"] + 32)
    out[pos["heap"] + 32:pos["heap"] + 32 + len(heap_data)] = heap_data
    groups = [names[:2], names[2:]]

    def tree(level, kids, last_names):
        node = b"TREE" + struct.pack("<BBHQQ", 0, level, len(kids), h5.UNDEF, h5.UNDEF) + struct.pack("<Q", 0)
        for kid, nm in zip(kids, last_names):
            node += struct.pack("<QQ", kid, off[nm])
        return node
    for at, node in ((pos["inner"], tree(1, [pos["leaf0"], pos["leaf1"]], [groups[0][-1], groups[1][-1]])),
                     (pos["leaf0"], tree(0, [pos["snod0"]], [groups[0][-1]])),
                     (pos["leaf1"], tree(0, [pos["snod1"]], [groups[1][-1]]))):
        out[at:at + len(node)] = node
    for g, at in zip(groups, (pos["snod0"], pos["snod1"])):
        s = b"SNOD" + struct.pack("<BBH", 1, 0, len(g)) + b"".join(
            struct.pack("<QQII16x", off[nm], pos[nm], 0, 0) for nm in g)
        out[at:at + len(s)] = s
    for nm in names:
        hdr = h5._object_header(msgs[nm])
        out[pos[nm]:pos[nm] + len(hdr)] = hdr
    # d_cont: the prefix counts all 4 messages (the continuation included); the second chunk holds 2
    struct.pack_into("<H", out, pos["d_cont"] + 2, 4)
    chunk = h5._object_header([(h5.MSG_DATASPACE, 0, h5._dataspace_msg((2,))),
                               (h5.MSG_LAYOUT, 1, struct.pack("<BBQQ", 3, 1, dpos["d_cont"], 16))])[16:]
    out[pos["cont"]:pos["cont"] + len(chunk)] = chunk
    for k in dpos:
        out[dpos[k]:dpos[k] + len(data[k])] = data[k]
    with open(path, "wb") as f:
        f.write(out)
    return expect


def test_h5_reader_format_variants(tmp_path):
    """Superblock 1, a two-level group B-tree, compact storage, big-endian types and an object
    header continued in a second chunk read back to the values written."""
    from vpm_gb300 import h5
    expect = _crafted_h5(str(tmp_path / "v.h5"))
    assert h5.keys(str(tmp_path / "v.h5")) == sorted(expect)
    got = h5.read(str(tmp_path / "v.h5"))
    for k, v in expect.items():
        assert got[k].shape == v.shape and got[k].dtype == v.dtype.newbyteorder("="), k
        np.testing.assert_array_equal(got[k], v)


def test_h5_reader_rejects_what_it_does_not_read(tmp_path):
    """A newer superblock and a non-HDF5 file raise, rather than read wrong values."""
    from vpm_gb300 import h5
    h5.write(str(tmp_path / "ok.h5"), {"a": np.zeros(2)})
    raw = bytearray((tmp_path / "ok.h5").read_bytes())
    raw[8] = 2                                            # superblock version 2
    (tmp_path / "v2.h5").write_bytes(bytes(raw))
    with pytest.raises(NotImplementedError):
        h5.read(str(tmp_path / "v2.h5"))
    (tmp_path / "no.h5").write_bytes(b"not an hdf5 file" * 4)
    with pytest.raises(ValueError):
        h5.read(str(tmp_path / "no.h5"))
