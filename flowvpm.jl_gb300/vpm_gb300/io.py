"""Particle-field files: the reference's `save` and `read!` (src/FLOWVPM_utils.jl:148-371,
494-571), writing and reading the same files.

Per saved step the reference writes `<name>.<nt>.h5` through HDF5.jl (:175-221): the scalar
datasets np, nt (int64) and t, and the float64 arrays X, Gamma, sigma, circulation, vol, static,
velocity, velocity_gradient_x/y/z, vorticity and, with an SFS model, C. Beside it,
`<name>.<nt>.xmf` is an XDMF 3 description of the same datasets for ParaView (:256-370). `save`
writes both, dataset for dataset and element for element, with `vpm_gb300.h5` (an HDF5 writer of
the original file format, which needs no HDF5 library). `read` is `read!`.

Array layout, as HDF5.jl stores the reference's Julia matrices: a 3-component field is an
np x 3 dataset in C order (each particle's three values contiguous), a scalar field np values.
`static` is float64, as the reference writes the particle matrix's row; its XDMF item still says
`Int`, as the reference's does.
"""
from __future__ import annotations

import os
import xml.etree.ElementTree as ET

import numpy as np

from . import h5
from .particlefield import (C_INDEX, CIRCULATION_INDEX, GAMMA_INDEX, J_INDEX, SIGMA_INDEX, STATIC_INDEX,
                            U_INDEX, VOL_INDEX, VORTICITY_INDEX, X_INDEX, ParticleField)

# (dataset, XDMF attribute name, rows of the particle matrix); the order and the names of
# src/FLOWVPM_utils.jl:192-221 (datasets) and :277-356 (attributes)
_VECTORS = (("Gamma", "Gamma", GAMMA_INDEX),
            ("velocity", "velocity", U_INDEX),
            ("velocity_gradient_x", "velocity gradient x", slice(J_INDEX.start, J_INDEX.start + 3)),
            ("velocity_gradient_y", "velocity gradient y", slice(J_INDEX.start + 3, J_INDEX.start + 6)),
            ("velocity_gradient_z", "velocity gradient z", slice(J_INDEX.start + 6, J_INDEX.start + 9)),
            ("vorticity", "vorticity", VORTICITY_INDEX))
_SCALARS = (("sigma", "sigma", SIGMA_INDEX),
            ("circulation", "circulation", CIRCULATION_INDEX),
            ("vol", "vol", VOL_INDEX))


def _data_item(parent, dims, h5fname: str, dataset: str, dtype: str = "Float"):
    el = ET.SubElement(parent, "DataItem", {"DataType": dtype, "Dimensions": dims, "Format": "HDF",
                                             "Precision": "8"})
    el.text = f"{h5fname}:{dataset}"
    return el


def save(pfield: ParticleField, file_name: str, *, path: str = "", add_num: bool = True, num: int = -1,
         createpath: bool = False, overwrite_time=None) -> str:
    """`save(pfield, file_name; path, add_num, num, createpath, overwrite_time)`,
    src/FLOWVPM_utils.jl:148-371: writes `<file_name>.<nt>.h5` and `<file_name>.<nt>.xmf`
    (`.<num>` when num >= 0, no number with add_num=False) and returns "<fname>.xmf;".
    An empty field is saved as one particle at the origin with zero strength and core
    size, as the reference does (:156-165)."""
    if pfield.get_np() == 0:
        dummy = ParticleField(1, nt=pfield.nt, t=pfield.t)
        dummy.add_particle((0.0, 0.0, 0.0), (0.0, 0.0, 0.0), 0.0)
        return save(dummy, file_name, path=path, add_num=add_num, num=num, createpath=createpath,
                    overwrite_time=overwrite_time)
    if createpath and path:
        os.makedirs(path, exist_ok=True)
    fname = file_name + ((f".{pfield.nt}" if num == -1 else f".{num}") if add_num else "")
    h5fname = fname + ".h5"
    n = pfield.get_np()
    time = overwrite_time if overwrite_time is not None else pfield.t
    time = int(time) if isinstance(time, (int, np.integer)) else float(time)   # an int stays int64
    P = pfield.particles

    # the datasets of src/FLOWVPM_utils.jl:179-221, in its order
    ds = {"np": int(n), "nt": int(pfield.nt),
          "t": time,
          "X": P[X_INDEX, :n].T, "Gamma": P[GAMMA_INDEX, :n].T, "sigma": P[SIGMA_INDEX, :n],
          "circulation": P[CIRCULATION_INDEX, :n], "vol": P[VOL_INDEX, :n],
          "static": P[STATIC_INDEX, :n]}
    for name, _, rows in _VECTORS[1:]:
        ds[name] = P[rows, :n].T
    les = pfield.isLES()
    if les:
        ds["C"] = P[C_INDEX, :n].T
    h5.write(os.path.join(path, h5fname), ds)

    # the XDMF of src/FLOWVPM_utils.jl:256-370
    xdmf = ET.Element("Xdmf", {"xmlns:xi": "http://www.w3.org/2001/XInclude", "Version": "3.0"})
    dom = ET.SubElement(xdmf, "Domain")
    grid = ET.SubElement(dom, "Grid", {"Name": "particles", "GridType": "Uniform"})
    ET.SubElement(grid, "Time", {"Value": repr(time)})
    geo = ET.SubElement(grid, "Geometry", {"Type": "XYZ"})
    _data_item(geo, f"{n} 3", h5fname, "X")
    ET.SubElement(grid, "Topology", {"Dimensions": str(n), "Type": "Polyvertex"})

    def attribute(dataset, name, typ, dims, dtype="Float"):
        at = ET.SubElement(grid, "Attribute", {"Center": "Node", "Name": name, "Type": typ})
        _data_item(at, dims, h5fname, dataset, dtype)
    for dataset, name, _ in _VECTORS:
        attribute(dataset, name, "Vector", f"{n} 3")
    for dataset, name, _ in _SCALARS:
        attribute(dataset, name, "Scalar", str(n))
    attribute("static", "static", "Scalar", str(n), "Int")
    if les:
        attribute("C", "C", "Vector", f"{n} 3")
    ET.indent(xdmf, space="\t")
    with open(os.path.join(path, fname + ".xmf"), "w") as f:
        f.write('<?xml version="1.0" encoding="utf-8"?>\n')
        f.write(ET.tostring(xdmf, encoding="unicode"))
        f.write("\n")
    return fname + ".xmf;"


def save_device(fld, file_name: str, *, les: bool = False, circulation=None, static=None, **kw) -> str:
    """`save` for the device-resident state (`vpm_gb300.device_step.DeviceField`): its x, gam,
    sig, vol, U and J (and C with les=True) are copied to a host particle matrix in the
    reference's rows and written by `save` (keywords as there).  The device state holds no
    circulation, static flags or vorticity: circulation and static are taken from the
    arguments (defaults 1 and 0, as `add_particle`'s), vorticity is written as zero."""
    n = int(fld.x.shape[0])
    pf = ParticleField(max(n, 1), nt=fld.nt, t=fld.t)
    host = lambda a: a.detach().to("cpu").double().numpy()
    P = pf.particles
    P[X_INDEX, :n] = host(fld.x).T
    P[GAMMA_INDEX, :n] = host(fld.gam).T
    P[SIGMA_INDEX, :n] = host(fld.sig)
    P[VOL_INDEX, :n] = host(fld.vol) if fld.vol is not None else 0.0
    P[CIRCULATION_INDEX, :n] = 1.0 if circulation is None else np.asarray(circulation, dtype=np.float64)
    P[STATIC_INDEX, :n] = 0.0 if static is None else np.asarray(static, dtype=np.float64)
    P[U_INDEX, :n] = host(fld.U).T
    P[J_INDEX, :n] = host(fld.J).T
    if les:
        P[C_INDEX, :n] = host(fld.C).T
        from .timeintegration import SFS_Cd_twolevel_nobackscatter
        pf.SFS = SFS_Cd_twolevel_nobackscatter   # marks the field as LES, so that C is written
    pf.np = n
    return save(pf, file_name, **kw)


def _datasets(xmf_path: str):
    """{dataset name: numpy array} of the DataItems of an XDMF file of `save`, each read from the
    `<file>.h5:<dataset>` it names."""
    root = ET.parse(xmf_path).getroot()
    base = os.path.dirname(xmf_path)
    out = {}
    for item in root.iter("DataItem"):
        fname, dataset = item.text.strip().rsplit(":", 1)
        a = h5.read(os.path.join(base, fname), [dataset])[dataset]
        dims = tuple(int(d) for d in item.get("Dimensions").split())
        if a.shape != dims:
            raise ValueError(f"{fname}:{dataset} has shape {a.shape}, the XDMF says {dims}")
        out[dataset] = a
    return out


def read(pfield: ParticleField, h5_fname: str, *, path: str = "", overwrite: bool = True,
         load_time: bool = True) -> ParticleField:
    """`read!(pfield, h5_fname; path, overwrite, load_time)`, src/FLOWVPM_utils.jl:494-571: loads
    X, Gamma, sigma, vol, circulation, static (if present, else 0) and C (if present, else 0) of
    `<h5_fname>.h5` after the field's particles (in their place with overwrite), and its time
    stamp t, nt with load_time."""
    if overwrite:
        pfield.np = 0
    h5fname = h5_fname if h5_fname.endswith(".h5") else h5_fname + ".h5"
    fpath = os.path.join(path, h5fname)
    names = h5.keys(fpath)
    want = ["np", "t", "nt", "X", "Gamma", "sigma", "vol", "circulation"]
    data = h5.read(fpath, want + [k for k in ("static", "C") if k in names])
    n = int(data["np"])
    if pfield.np + n > pfield.maxparticles:
        raise RuntimeError(f"The field to be read ({h5_fname}) contains {n} particles but max number of "
                           f"particles is {pfield.maxparticles}.")
    if load_time:
        pfield.t = data["t"].item()
        pfield.nt = int(data["nt"])
    sl = slice(pfield.np, pfield.np + n)
    P = pfield.particles
    P[X_INDEX, sl] = data["X"].T
    P[GAMMA_INDEX, sl] = data["Gamma"].T
    P[SIGMA_INDEX, sl] = data["sigma"]
    P[VOL_INDEX, sl] = data["vol"]
    P[CIRCULATION_INDEX, sl] = data["circulation"]
    if "static" in data:
        st = data["static"]
        if not np.all((st == 0) | (st == 1)):           # the reference converts them to Bool
            raise ValueError(f"static flags of {h5_fname} other than 0 and 1")
        P[STATIC_INDEX, sl] = st.astype(np.float64)
    else:
        P[STATIC_INDEX, sl] = 0.0
    P[C_INDEX, sl] = data["C"].T if "C" in data else 0.0
    pfield.np += n
    return pfield
