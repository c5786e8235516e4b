"""Particle-field files (vpm_gb300.io): the reference's save / read! (src/FLOWVPM_utils.jl:148-371,
494-571) with the XDMF the reference writes and a raw binary file in place of HDF5. CPU only."""
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
    assert os.path.exists(tmp_path / "field.17.xmf") and os.path.exists(tmp_path / "field.17.bin")
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
    for a in grid.findall("Attribute"):
        item = a.find("DataItem")
        assert item.get("Format") == "Binary" and item.get("Precision") == "8"
        assert item.get("DataType") == ("Int" if a.get("Name") == "static" else "Float")
        assert item.text == "f.3.bin"


def test_binary_datasets_at_their_offsets(tmp_path):
    pf = _field(33)
    vio.save(pf, "g", path=str(tmp_path), add_num=False)
    raw = (tmp_path / "g.bin").read_bytes()
    grid = ET.parse(tmp_path / "g.xmf").getroot().find("Domain/Grid")
    n = pf.np

    def at(name):
        item = (grid.find("Geometry/DataItem") if name == "X" else
                next(a for a in grid.findall("Attribute") if a.get("Name") == name).find("DataItem"))
        dims = [int(d) for d in item.get("Dimensions").split()]
        off = int(item.get("Seek"))
        dt = "<f8" if item.get("DataType") == "Float" else "<i8"
        return np.frombuffer(raw[off:off + 8 * int(np.prod(dims))], dtype=dt).reshape(dims)
    P = pf.particles
    np.testing.assert_array_equal(at("X"), P[0:3, :n].T)
    np.testing.assert_array_equal(at("velocity gradient y"), P[J_INDEX.start + 3:J_INDEX.start + 6, :n].T)
    np.testing.assert_array_equal(at("vorticity"), P[VORTICITY_INDEX, :n].T)
    np.testing.assert_array_equal(at("static"), P[STATIC_INDEX, :n].astype(np.int64))
    assert len(raw) == 8 * n * (3 * 7 + 4)      # X, 6 vector attributes, 4 scalars; no C without SFS


def test_empty_field_saves_one_dummy_particle(tmp_path):
    pf = vpm.ParticleField(10, nt=4, t=0.5)
    vio.save(pf, "e", path=str(tmp_path))
    back = vio.read(vpm.ParticleField(2), "e.4", path=str(tmp_path))
    assert back.np == 1 and back.nt == 4 and back.t == 0.5
    np.testing.assert_array_equal(back.particles[0:7, 0], 0.0)


def test_read_overflow_and_append(tmp_path):
    pf = _field(20)
    vio.save(pf, "h", path=str(tmp_path))
    with pytest.raises(RuntimeError, match="max number of particles"):
        vio.read(vpm.ParticleField(19), "h.17", path=str(tmp_path))
    two = vpm.ParticleField(40)
    vio.read(two, "h.17", path=str(tmp_path))
    vio.read(two, "h.17.xmf", path=str(tmp_path), overwrite=False, load_time=False)
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
    data, _ = vio._datasets(str(tmp_path / "dev.9.xmf"))
    np.testing.assert_array_equal(data["velocity_gradient_z"], fld.J.numpy()[:, 6:9])
