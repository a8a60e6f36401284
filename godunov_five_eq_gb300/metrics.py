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
