"""Output path of the solver loop: the datasets that
SolverGodunovFiveEq::save_solution_hdf5 (SolverGodunovFiveEq.cpp:771-955)
writes, selected and named as it selects and names them, packed on the device
by g5_pack_fields (one pass over the state, one device-to-host copy) and
written with an XDMF description.

The reference hands its datasets to kalypsso-core's HDF5_Xdmf_Writer, a
library outside the reference tree whose file layout is not restated here.
This module writes, per output, one raw little-endian float64 file holding
the datasets one after the other (each [n_owned blocks][bsize^dim cells], the
block table's order, x fastest within a block) and an XDMF 3 file describing
every owned block as a uniform cell-centred grid with its datasets located
inside the raw file.
"""
from __future__ import annotations

import os
from xml.sax.saxutils import quoteattr

import numpy as np

FIELD_DERIVED = 64
MAX_PACK_FIELDS = 16
# ComputeDerivedQuantities' DERIVED_QUANTITY enum (utils/ComputeDerivedQuantities.h:45-54)
DERIVED_QUANTITIES = ("RHO_MIX", "THERMAL_PRESSURE", "SPEED_OF_SOUND", "SPECIFIC_EKIN", "LOCAL_MACH_NUMBER", "VX", "VY", "VZ")


def hydro_names(dim: int) -> tuple:
    """FiveEq<dim>::get_var_names for the hydrodynamic variables ID, IE, IU,
    IV[, IW] (models/FiveEq.h:123-137)."""
    return ("rho_mix", "e_tot", "rho_vx", "rho_vy") + (("rho_vz",) if dim == 3 else ())


def var_name(dim: int, var: int) -> str:
    """FiveEq<dim>::name (models/FiveEq.h:93-102): the hydrodynamic names, then
    alpha_<mat> and alpha_rho_<mat> for the per-material pairs."""
    names = hydro_names(dim)
    hydro = len(names)
    if var < hydro:
        return names[var]
    i_mat, i_var = divmod(var - hydro, 2)
    return ("alpha", "alpha_rho")[i_var] + "_" + str(i_mat)


def select_fields(dim: int, nmat: int, write_variables=(), checkpoint: bool = False, pure_checkpoint: bool = False) -> list:
    """The datasets of one output as save_solution_hdf5 picks them
    (SolverGodunovFiveEq.cpp:809-886), in its order, as (name, code) pairs:
    code < nv a variable of the state (the reference's VarId), FIELD_DERIVED
    + q the derived quantity q.

    * every hydrodynamic variable that write_variables names, or all of them
      at a checkpoint;
    * per material i < nmat ("run/nmat"): alpha_i then alpha_rho_i, the same
      rule;
    * unless pure_checkpoint: each derived quantity whose lower-case enum name
      write_variables lists, rho_mix excepted (already a variable).
    "rho_mix_schlieren" (kalypsso-core's ComputeSchlieren) is not produced
    here and raises.
    """
    wv = list(write_variables)
    hydro = len(hydro_names(dim))
    if nmat < 0 or nmat > 2:
        raise ValueError(f"nmat={nmat}: the state holds two materials")
    out = []
    for v in range(hydro):
        name = var_name(dim, v)
        if name in wv or checkpoint:
            out.append((name, v))
    for i_mat in range(nmat):
        for v in (hydro + 2 * i_mat, hydro + 1 + 2 * i_mat):
            name = var_name(dim, v)
            if name in wv or checkpoint:
                out.append((name, v))
    if not pure_checkpoint:
        if "rho_mix_schlieren" in wv:
            raise NotImplementedError("rho_mix_schlieren: kalypsso-core's ComputeSchlieren is not part of this library")
        for q, enum_name in enumerate(DERIVED_QUANTITIES):
            name = enum_name.lower()
            if name in wv and name != "rho_mix":
                out.append((name, FIELD_DERIVED + q))
    return out


def pack(impl, U, codes, stream=None) -> np.ndarray:
    """The datasets `codes` of the owned blocks of U (device), packed on the
    device by g5_pack_fields in launches of up to 16 fields: host array
    [len(codes), n_owned, ncell]."""
    import torch

    t = impl.table
    dev = torch.empty((len(codes), t.n_owned, t.ncell), dtype=torch.float64, device=U.device)
    for k in range(0, len(codes), MAX_PACK_FIELDS):
        chunk = codes[k : k + MAX_PACK_FIELDS]
        impl.pack_fields(U, chunk, 0, t.n_owned, out=dev[k : k + len(chunk)], stream=stream)
    host = torch.empty(dev.shape, dtype=torch.float64, pin_memory=True)
    host.copy_(dev, non_blocking=True)
    (stream or torch.cuda.current_stream()).synchronize()
    return host.numpy()


def write_xdmf(out_dir: str, basename: str, table, names, data: np.ndarray, time: float = 0.0, iteration: int = 0) -> dict:
    """Write <basename>.bin (data as little-endian float64, [field][block][cell])
    and <basename>.xmf (a spatial collection of one uniform grid per owned
    block: origin coord * bsize * dx(level), spacing dx(level), the fields as
    cell attributes at their offsets in the raw file).  Returns the paths and
    the byte count of the raw file."""
    dim, b, n = table.dim, table.bsize, table.n_owned
    data = np.ascontiguousarray(data, dtype="<f8")
    if data.shape != (len(names), n, b**dim):
        raise ValueError(f"data shape {data.shape} != {(len(names), n, b ** dim)}")
    os.makedirs(out_dir, exist_ok=True)
    bin_name = basename + ".bin"
    bin_path = os.path.join(out_dir, bin_name)
    data.tofile(bin_path)
    cell_dims = " ".join([str(b)] * dim)  # z y x (XDMF order), all equal
    node_dims = " ".join([str(b + 1)] * dim)
    topo = "3DCoRectMesh" if dim == 3 else "2DCoRectMesh"
    geo = "ORIGIN_DXDYDZ" if dim == 3 else "ORIGIN_DXDY"
    block_bytes = b**dim * 8
    lines = [
        '<?xml version="1.0" ?>',
        '<Xdmf Version="3.0">',
        "  <Domain>",
        '    <Grid Name="blocks" GridType="Collection" CollectionType="Spatial">',
        f'      <Time Value="{float(time)!r}"/>',
        f'      <Information Name="iteration" Value="{int(iteration)}"/>',
    ]
    for j in range(n):
        L = int(table.level[j])
        dx = float(table.level_dx[L])
        origin = [float(table.coord[j, e]) * b * dx for e in range(dim)][::-1]  # z y x
        spacing = [dx] * dim
        lines.append(f'      <Grid Name="block_{j}" GridType="Uniform">')
        lines.append(f'        <Information Name="level" Value="{L}"/>')
        lines.append(f'        <Topology TopologyType="{topo}" Dimensions="{node_dims}"/>')
        lines.append(f'        <Geometry GeometryType="{geo}">')
        lines.append(f'          <DataItem Format="XML" Dimensions="{dim}">{" ".join(repr(o) for o in origin)}</DataItem>')
        lines.append(f'          <DataItem Format="XML" Dimensions="{dim}">{" ".join(repr(s) for s in spacing)}</DataItem>')
        lines.append("        </Geometry>")
        for k, name in enumerate(names):
            seek = (k * n + j) * block_bytes
            lines.append(f"        <Attribute Name={quoteattr(name)} AttributeType=\"Scalar\" Center=\"Cell\">")
            lines.append(
                f'          <DataItem Format="Binary" Endian="Little" NumberType="Float" Precision="8" Seek="{seek}" '
                f'Dimensions="{cell_dims}">{bin_name}</DataItem>'
            )
            lines.append("        </Attribute>")
        lines.append("      </Grid>")
    lines += ["    </Grid>", "  </Domain>", "</Xdmf>", ""]
    xmf_path = os.path.join(out_dir, basename + ".xmf")
    with open(xmf_path, "w") as f:
        f.write("\n".join(lines))
    return {"xmf": xmf_path, "bin": bin_path, "bytes": int(data.nbytes)}


def save_solution(impl, U, out_dir: str, basename: str, write_variables=(), nmat: int = 2, checkpoint: bool = False,
                  pure_checkpoint: bool = False, time: float = 0.0, iteration: int = 0, stream=None) -> dict:
    """save_solution_hdf5's dataset path for the state U (device) of the
    context's mesh: select, pack on the device, write.  Returns the paths,
    the byte count and the dataset names."""
    sel = select_fields(impl.table.dim, nmat, write_variables, checkpoint, pure_checkpoint)
    if not sel:
        raise ValueError("no dataset selected")
    names = [s[0] for s in sel]
    data = pack(impl, U, [s[1] for s in sel], stream=stream)
    res = write_xdmf(out_dir, basename, impl.table, names, data, time, iteration)
    res["names"] = names
    return res
