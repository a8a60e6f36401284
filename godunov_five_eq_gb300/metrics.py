"""Error norms used to compare the mixed-precision path with the FP64 method."""
import numpy as np

from .configs import ids


def l1_relative(table, A, B):
    """Volume-weighted relative L1 error per conservative variable of A against B.

    err_v = sum_cells V |A_v - B_v| / sum_cells V |B_v|, except for the
    momentum components, whose denominator is sum_cells V |rho u| (magnitude
    of the momentum vector of B), so that a component that vanishes in B
    does not turn round-off into a large relative error.
    """
    n = table.n_owned
    I = ids(table.dim)
    vol = table.level_dx[table.level[:n]] ** table.dim
    mom = [I["IU"], I["IV"]] + ([I["IW"]] if table.dim == 3 else [])
    mag = np.sqrt(sum(B[:n, m] ** 2 for m in mom))
    out = []
    for v in range(table.nv):
        num = (np.abs(A[:n, v] - B[:n, v]).sum(axis=1) * vol).sum()
        ref = mag if v in mom else np.abs(B[:n, v])
        den = (ref.sum(axis=1) * vol).sum()
        out.append(float(num / den) if den > 0 else float(num))
    return np.array(out)


def linf_relative(table, A, B):
    """Relative L-infinity error per conservative variable of A against B:
    max |A_v - B_v| / max |B_v| (momentum components: / max |rho u|)."""
    n = table.n_owned
    I = ids(table.dim)
    mom = [I["IU"], I["IV"]] + ([I["IW"]] if table.dim == 3 else [])
    mag = np.sqrt(sum(B[:n, m] ** 2 for m in mom))
    out = []
    for v in range(table.nv):
        num = np.abs(A[:n, v] - B[:n, v]).max()
        den = (mag if v in mom else np.abs(B[:n, v])).max()
        out.append(float(num / den) if den > 0 else float(num))
    return np.array(out)


def material_masses(table, U):
    """Total mass of each material: sum over owned cells of alpha_k rho_k x cell volume."""
    n = table.n_owned
    I = ids(table.dim)
    vol = table.level_dx[table.level[:n]] ** table.dim
    return np.array([float((U[:n, I[k]].sum(axis=1) * vol).sum()) for k in ("IAD0", "IAD1")])


def cell_centres(table):
    """Cell-centre coordinates [n_owned, dim, ncell] from the block table alone."""
    b, dim, n = table.bsize, table.dim, table.n_owned
    idx = np.arange(b**dim)
    loc = [idx % b, (idx // b) % b, idx // (b * b)]
    dx = table.level_dx[table.level[:n]][:, None]
    return np.stack([(table.coord[:n, e][:, None] * b + loc[e][None, :] + 0.5) * dx for e in range(dim)], axis=1)


def interface_metrics(table, U, material=1):
    """Region of `material` (volume fraction > 0.5): its volume, centroid and
    bounding box of cell centres (the alpha = 0.5 contour's position)."""
    n = table.n_owned
    I = ids(table.dim)
    a = U[:n, I["IA0"]] if material == 0 else U[:n, I["IA1"]]
    vol = np.broadcast_to(table.level_dx[table.level[:n]][:, None] ** table.dim, a.shape)
    xc = cell_centres(table)
    sel = a > 0.5
    v = float(vol[sel].sum())
    if v == 0.0:
        return {"volume": 0.0, "centroid": None, "extent": None}
    cen = [float((xc[:, e][sel] * vol[sel]).sum() / v) for e in range(table.dim)]
    ext = [[float(xc[:, e][sel].min()), float(xc[:, e][sel].max())] for e in range(table.dim)]
    return {"volume": v, "centroid": cen, "extent": ext}


def interface_error(table, A, B, material=1):
    """Position error of the material-region of A against B: relative volume
    difference, centroid distance and the largest bounding-box edge shift."""
    ma, mb = interface_metrics(table, A, material), interface_metrics(table, B, material)
    if ma["centroid"] is None or mb["centroid"] is None:
        return None
    dcen = float(np.sqrt(sum((x - y) ** 2 for x, y in zip(ma["centroid"], mb["centroid"]))))
    dext = float(max(abs(p - q) for ea, eb in zip(ma["extent"], mb["extent"]) for p, q in zip(ea, eb)))
    return {
        "volume_rel_diff": abs(ma["volume"] - mb["volume"]) / mb["volume"],
        "centroid_distance": dcen,
        "extent_max_shift": dext,
        "finest_dx": float(table.level_dx[table.level[: table.n_owned].max()]),
    }
