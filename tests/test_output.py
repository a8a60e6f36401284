"""Output path (SolverGodunovFiveEq::save_solution_hdf5, SolverGodunovFiveEq.cpp:771-955).

CPU: the dataset names and selection rules against the reference's code
(models/FiveEq.h:93-137, SolverGodunovFiveEq.cpp:809-886), and the XDMF +
raw writer read back (every block's origin, spacing and every dataset at its
offset).  GPU: g5_pack_fields bit-exact against the state's variables and
the oracle's derived quantities, 2D and 3D, and a written output read back.
"""
import os
import xml.etree.ElementTree as ET

import numpy as np
import pytest

from godunov_five_eq_gb300 import output
from godunov_five_eq_gb300.mesh import cell_centers
from tests.helpers import amr_mesh, smooth_state, water_air_params


def test_variable_names_follow_the_model():
    # FiveEq<dim>::name: the hydrodynamic names, then alpha_i / alpha_rho_i
    assert [output.var_name(2, v) for v in range(8)] == [
        "rho_mix", "e_tot", "rho_vx", "rho_vy", "alpha_0", "alpha_rho_0", "alpha_1", "alpha_rho_1"]
    assert [output.var_name(3, v) for v in range(9)] == [
        "rho_mix", "e_tot", "rho_vx", "rho_vy", "rho_vz", "alpha_0", "alpha_rho_0", "alpha_1", "alpha_rho_1"]


def test_selection_rules():
    # a checkpoint writes every variable, the materials' pairs in material order
    sel = output.select_fields(2, 2, (), checkpoint=True)
    assert sel == [(output.var_name(2, v), v) for v in (0, 1, 2, 3, 4, 5, 6, 7)]
    # otherwise the listed ones, in the writer's order (not the list's)
    sel = output.select_fields(3, 2, ["alpha_1", "rho_vz", "rho_mix", "speed_of_sound", "vx"])
    assert [s[0] for s in sel] == ["rho_mix", "rho_vz", "alpha_1", "speed_of_sound", "vx"]
    assert sel[3] == ("speed_of_sound", output.FIELD_DERIVED + 2) and sel[4] == ("vx", output.FIELD_DERIVED + 5)
    # "run/nmat" bounds the materials written
    assert [s[0] for s in output.select_fields(2, 1, (), checkpoint=True)][-2:] == ["alpha_0", "alpha_rho_0"]
    assert output.select_fields(2, 0, ["alpha_0"]) == []
    # rho_mix is a variable, never a derived dataset; a pure checkpoint has no derived ones
    assert output.select_fields(2, 2, ["rho_mix"]) == [("rho_mix", 0)]
    assert output.select_fields(2, 2, ["thermal_pressure"], checkpoint=True, pure_checkpoint=True)[-1] == ("alpha_rho_1", 7)
    with pytest.raises(NotImplementedError):
        output.select_fields(2, 2, ["rho_mix_schlieren"])
    with pytest.raises(ValueError):
        output.select_fields(2, 3, ())


def _read_back(res, names, table):
    root = ET.parse(res["xmf"]).getroot()
    grids = root.find("Domain").find("Grid").findall("Grid")
    assert len(grids) == table.n_owned
    raw = np.fromfile(res["bin"], dtype="<f8")
    b, dim = table.bsize, table.dim
    got = np.zeros((len(names), table.n_owned, b**dim))
    origins = np.zeros((table.n_owned, dim))
    spacing = np.zeros(table.n_owned)
    for j, g in enumerate(grids):
        items = g.find("Geometry").findall("DataItem")
        origins[j] = [float(x) for x in items[0].text.split()][::-1]
        spacing[j] = float(items[1].text.split()[0])
        attrs = g.findall("Attribute")
        assert [a.get("Name") for a in attrs] == names
        for k, a in enumerate(attrs):
            d = a.find("DataItem")
            assert d.get("Center") is None and a.get("Center") == "Cell"
            off = int(d.get("Seek")) // 8
            got[k, j] = raw[off : off + b**dim]
    return got, origins, spacing


@pytest.mark.parametrize("dim", [2, 3])
def test_xdmf_writer_reads_back(tmp_path, dim):
    mesh, t = amr_mesh(dim=dim, b=8, nref=2, seed=dim)
    names = ["rho_mix", "alpha_0", "vx"]
    data = np.random.default_rng(dim).standard_normal((3, t.n_owned, t.ncell))
    res = output.write_xdmf(str(tmp_path), "out_0001", t, names, data, time=0.25, iteration=17)
    assert os.path.getsize(res["bin"]) == data.nbytes == res["bytes"]
    got, origins, spacing = _read_back(res, names, t)
    assert np.array_equal(got, data)
    # block geometry: the first cell centre is origin + dx / 2
    cc = cell_centers(mesh, t)
    assert np.allclose(origins + 0.5 * spacing[:, None], cc[:, :, 0], rtol=0, atol=1e-14)
    assert np.allclose(spacing, t.level_dx[t.level[: t.n_owned]], rtol=0, atol=0)
    root = ET.parse(res["xmf"]).getroot()
    assert float(root.find("Domain").find("Grid").find("Time").get("Value")) == 0.25


@pytest.mark.gpu
@pytest.mark.parametrize("dim", [2, 3])
def test_gpu_pack_fields_bit_exact(tmp_path, dim):
    torch = pytest.importorskip("torch")
    from godunov_five_eq_gb300.implem import GodunovImplemGB300
    from oracle import oracle as orc

    mesh, t = amr_mesh(dim=dim, b=8, nref=2, seed=dim)
    p = water_air_params(t, dim=dim, b=8)
    U = smooth_state(mesh, t, p, seed=dim)
    impl = GodunovImplemGB300(p, t)
    A = torch.from_numpy(U).cuda()
    n = t.n_owned
    # every variable and every derived quantity (17 fields in 3D: two launches)
    codes = list(range(t.nv)) + [output.FIELD_DERIVED + q for q in range(8)]
    got = output.pack(impl, A, codes)
    for k, c in enumerate(codes):
        if c < t.nv:
            assert np.array_equal(got[k], U[:n, c]), c
        else:
            ref = orc.derived(p, U, orc.DERIVED_QUANTITIES[c - output.FIELD_DERIVED], 0, n)[:n, 0]
            assert np.array_equal(got[k], ref), c
    # a block range
    part = impl.pack_fields(A, [1, output.FIELD_DERIVED + 1], 3, 5).cpu().numpy()
    assert np.array_equal(part[0], U[3:8, 1]) and np.array_equal(part[1], got[t.nv + 1, 3:8])
    # a whole output written and read back
    res = output.save_solution(impl, A, str(tmp_path), "ckpt", ["thermal_pressure"], nmat=2, checkpoint=True, time=1.0, iteration=3)
    back, _, _ = _read_back(res, res["names"], t)
    assert res["names"][-1] == "thermal_pressure"
    assert np.array_equal(back[: t.nv], np.moveaxis(U[:n], 1, 0))
    impl.close()
