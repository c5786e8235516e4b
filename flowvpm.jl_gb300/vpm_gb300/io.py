"""Particle-field files: the reference's `save` and `read!` (src/FLOWVPM_utils.jl:148-371,
494-571), with the datasets in a raw binary file instead of HDF5.

The reference writes, per saved step, `<name>.<nt>.h5` (the scalars np, nt, t and the datasets
X, Gamma, sigma, circulation, vol, static, velocity, velocity_gradient_x/y/z, vorticity and,
with an SFS model, C; :179-221) and `<name>.<nt>.xmf`, an XDMF 3 description of the same
datasets for ParaView (:256-370). No HDF5 library exists to this package, so `save` writes the
same XDMF, element for element and name for name, with every DataItem pointing into one raw
little-endian binary file `<name>.<nt>.bin` (`Format="Binary"`, a byte offset in `Seek`)
instead of `<name>.<nt>.h5:/<dataset>`; the scalars np, nt and t also go into `Information`
elements of the grid. ParaView's XDMF reader takes binary DataItems as it takes HDF ones.
`read` is `read!` for these files (the reference's `read!` itself reads only `.h5`).

Array layout, as in the reference's HDF5 datasets: a 3-component field is np x 3 in C order
(each particle's three values contiguous), a scalar field is np values; FP64 throughout, and
`static` as 64-bit integers (the reference's XDMF declares it `Int`, precision 8).
"""
from __future__ import annotations

import os
import xml.etree.ElementTree as ET

import numpy as np

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


def _data_item(parent, dims, offset: int, binname: str, dtype: str = "Float"):
    el = ET.SubElement(parent, "DataItem", {"DataType": dtype, "Dimensions": dims, "Format": "Binary",
                                             "Endian": "Little", "Precision": "8", "Seek": str(offset)})
    el.text = binname
    return el


def save(pfield: ParticleField, file_name: str, *, path: str = "", add_num: bool = True, num: int = -1,
         createpath: bool = False, overwrite_time=None) -> str:
    """`save(pfield, file_name; path, add_num, num, createpath, overwrite_time)`,
    src/FLOWVPM_utils.jl:148-371: writes `<file_name>.<nt>.xmf` and `<file_name>.<nt>.bin`
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
    binname = fname + ".bin"
    n = pfield.get_np()
    time = float(overwrite_time) if overwrite_time is not None else float(pfield.t)
    P = pfield.particles

    # the datasets, in the reference's order, and their byte offsets
    blocks, offsets, off = [], {}, 0

    def put(name, arr):
        nonlocal off
        a = np.ascontiguousarray(arr)
        offsets[name] = off
        blocks.append(a.astype("<f8" if a.dtype.kind == "f" else "<i8", copy=False).tobytes())
        off += len(blocks[-1])
    put("X", P[X_INDEX, :n].T)
    put("Gamma", P[GAMMA_INDEX, :n].T)
    put("sigma", P[SIGMA_INDEX, :n])
    put("circulation", P[CIRCULATION_INDEX, :n])
    put("vol", P[VOL_INDEX, :n])
    put("static", P[STATIC_INDEX, :n].astype(np.int64))
    for ds, _, rows in _VECTORS[1:]:
        put(ds, P[rows, :n].T)
    les = pfield.isLES()
    if les:
        put("C", P[C_INDEX, :n].T)
    with open(os.path.join(path, binname), "wb") as f:
        for b in blocks:
            f.write(b)

    # the XDMF of src/FLOWVPM_utils.jl:256-370, binary DataItems
    xdmf = ET.Element("Xdmf", {"xmlns:xi": "http://www.w3.org/2001/XInclude", "Version": "3.0"})
    dom = ET.SubElement(xdmf, "Domain")
    grid = ET.SubElement(dom, "Grid", {"Name": "particles", "GridType": "Uniform"})
    for k, v in (("np", n), ("nt", pfield.nt), ("t", repr(time))):
        ET.SubElement(grid, "Information", {"Name": k, "Value": str(v)})
    ET.SubElement(grid, "Time", {"Value": repr(time)})
    geo = ET.SubElement(grid, "Geometry", {"Type": "XYZ"})
    _data_item(geo, f"{n} 3", offsets["X"], binname)
    ET.SubElement(grid, "Topology", {"Dimensions": str(n), "Type": "Polyvertex"})

    def attribute(ds, name, typ, dims, dtype="Float"):
        at = ET.SubElement(grid, "Attribute", {"Center": "Node", "Name": name, "Type": typ})
        _data_item(at, dims, offsets[ds], binname, dtype)
    for ds, name, _ in _VECTORS:
        attribute(ds, name, "Vector", f"{n} 3")
    for ds, name, _ in _SCALARS:
        attribute(ds, name, "Scalar", str(n))
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
    """{dataset name: numpy array} and the grid's Information values of a file of `save`."""
    root = ET.parse(xmf_path).getroot()
    grid = root.find("Domain/Grid")
    info = {el.get("Name"): el.get("Value") for el in grid.findall("Information")}
    base = os.path.dirname(xmf_path)
    names = {name: ds for ds, name, _ in _VECTORS + _SCALARS}
    names.update({"static": "static", "C": "C"})
    items = [("X", grid.find("Geometry/DataItem"))]
    items += [(names[at.get("Name")], at.find("DataItem")) for at in grid.findall("Attribute")]
    out = {}
    for ds, item in items:
        dims = [int(d) for d in item.get("Dimensions").split()]
        dtype = "<f8" if item.get("DataType") == "Float" else "<i8"
        with open(os.path.join(base, item.text.strip()), "rb") as f:
            f.seek(int(item.get("Seek", "0")))
            a = np.frombuffer(f.read(8 * int(np.prod(dims))), dtype=dtype)
        out[ds] = a.reshape(dims)
    return out, info


def read(pfield: ParticleField, fname: str, *, path: str = "", overwrite: bool = True,
         load_time: bool = True) -> ParticleField:
    """`read!(pfield, fname; path, overwrite, load_time)`, src/FLOWVPM_utils.jl:494-571, for a
    file of `save`: loads X, Gamma, sigma, vol, circulation, static (if present) and C (else
    zero) after the field's particles (or in their place with overwrite), and the time stamp."""
    if overwrite:
        pfield.np = 0
    xmf = fname if fname.endswith(".xmf") else fname + ".xmf"
    data, info = _datasets(os.path.join(path, xmf))
    n = int(info["np"])
    if pfield.np + n > pfield.maxparticles:
        raise RuntimeError(f"The field to be read ({fname}) contains {n} particles but max number of "
                           f"particles is {pfield.maxparticles}.")
    if load_time:
        pfield.t = float(info["t"])
        pfield.nt = int(info["nt"])
    sl = slice(pfield.np, pfield.np + n)
    P = pfield.particles
    P[X_INDEX, sl] = data["X"].T
    P[GAMMA_INDEX, sl] = data["Gamma"].T
    P[SIGMA_INDEX, sl] = data["sigma"]
    P[VOL_INDEX, sl] = data["vol"]
    P[CIRCULATION_INDEX, sl] = data["circulation"]
    P[STATIC_INDEX, sl] = data["static"].astype(np.float64) if "static" in data else 0.0
    P[C_INDEX, sl] = data["C"].T if "C" in data else 0.0
    pfield.np += n
    return pfield
