"""NumPy restatements of the reference's RawModule kernels (FP64).

Each function follows the CUDA-C kernel it names, term by term and in the same
summation order, over the whole ``ny x nx`` field instead of one thread per
point.  Wrap-around neighbours use ``np.roll`` (``np.roll(a, -1, 1)[i, j] ==
a[i, (j+1) % nx]``), matching the manual wrap at +-1, +-2 in the kernels.
"""
import numpy as np


def _flat(a):
    """Flat view of a kernel argument (1-D views or whole 2-D buffers)."""
    v = a.reshape(-1)
    assert v.base is a or v is a or np.shares_memory(v, a)
    return v


def _field(a, nx, ny):
    return _flat(a)[: nx * ny].reshape(ny, nx)


def _neighbour_sums(a):
    """(sum of +-1 neighbours, sum of +-2 neighbours), in the kernels' order:
    x+1, x-1, y+1, y-1 (and the same at distance 2)."""
    t1 = np.roll(a, -1, 1) + np.roll(a, 1, 1) + np.roll(a, -1, 0) + np.roll(a, 1, 0)
    t2 = np.roll(a, -2, 1) + np.roll(a, 2, 1) + np.roll(a, -2, 0) + np.roll(a, 2, 0)
    return t1, t2


def lapg(inp, out, nx, ny, c2, c3):
    """core/seis_forward2.py:382-421: 4th-order Laplacian without the centre."""
    nx, ny = int(nx), int(ny)
    t1, t2 = _neighbour_sums(_field(inp, nx, ny))
    _flat(out)[: nx * ny] = (c2 * t1 + c3 * t2).ravel()


def update_p(temp1, temp2, alpha, pout, pout1, pout2, lapg_store, nx, ny, it,
             src_idx, s_mod):
    """core/seis_forward2.py:429-462: leapfrog update + source injection."""
    n = int(nx) * int(ny)
    temp1, temp2, alpha, pout, pout1, pout2, lapg_store = (
        _flat(a)[:n] for a in (temp1, temp2, alpha, pout, pout1, pout2, lapg_store))
    out = temp1 * pout1 - temp2 * pout + alpha * lapg_store
    out[int(src_idx[0])] += s_mod[int(it)]
    pout2[:] = out


def update_p_diff(temp1, temp1_diff, temp2, temp2_diff, alpha, alpha_diff,
                  pout, pout1, pout2, lapg_store, lapg_store_diff,
                  pout_diff, pout1_diff, pout2_diff, nx, ny, it, src_idx,
                  s_mod_diff):
    """core/seis_forward2.py:470-509: tangent (Born) update."""
    n = int(nx) * int(ny)
    (temp1, temp1_diff, temp2, temp2_diff, alpha, alpha_diff, pout, pout1, lapg_store,
     lapg_store_diff, pout_diff, pout1_diff, pout2_diff) = (
        _flat(a)[:n] for a in (temp1, temp1_diff, temp2, temp2_diff, alpha, alpha_diff, pout,
                               pout1, lapg_store, lapg_store_diff, pout_diff, pout1_diff, pout2_diff))
    out = (temp1_diff * pout1 + temp1 * pout1_diff
           - temp2_diff * pout - temp2 * pout_diff
           + alpha_diff * lapg_store + alpha * lapg_store_diff)
    out[int(src_idx[0])] += s_mod_diff[int(it)]
    pout2_diff[:] = out


def update_p_adjoint(temp1, temp2, alpha, p_complete1, p_complete2, lapg_store,
                     s_mod_adjoint, adj1, adj2, adj3, temp1_adjoint,
                     temp2_adjoint, alpha_adjoint, lapg_store_adjoint,
                     nx, ny, it, c2, c3, src_idx):
    """core/seis_forward2.py:517-579: one reverse step with lapg^T folded in."""
    nx, ny = int(nx), int(ny)
    n = nx * ny
    t1, t2 = _neighbour_sums(_field(alpha, nx, ny) * _field(adj3, nx, ny))
    (temp1, temp2, p_complete1, p_complete2, lapg_store, adj1, adj2, q3, temp1_adjoint,
     temp2_adjoint, alpha_adjoint) = (
        _flat(a)[:n] for a in (temp1, temp2, p_complete1, p_complete2, lapg_store, adj1, adj2,
                               adj3, temp1_adjoint, temp2_adjoint, alpha_adjoint))
    s_mod_adjoint[int(it)] = q3[int(src_idx[0])]
    adj2 += temp1 * q3
    temp1_adjoint += p_complete2 * q3
    adj1 -= temp2 * q3
    temp2_adjoint -= p_complete1 * q3
    alpha_adjoint += lapg_store * q3
    adj2 += (c2 * t1 + c3 * t2).ravel()


def _tree_dot(a, b, block=1024):
    """Block-strided partial sums followed by the shared-memory tree reduction
    of the single-block L-BFGS kernels (core/seis_numerics.py:465-483)."""
    n = a.shape[0]
    part = np.zeros(block)
    chunk = (n + block - 1) // block
    for c in range(chunk):
        lo = c * block
        hi = min(lo + block, n)
        part[: hi - lo] += a[lo:hi] * b[lo:hi]
    stride = block >> 1
    while stride > 0:
        part[:stride] += part[stride: 2 * stride]
        stride >>= 1
    return part[0]


def lbfgs_backward(old_stps, old_dirs, ro, q, al, num_old, n):
    """core/seis_numerics.py:451-501."""
    n = int(n)
    for i in range(int(num_old) - 1, -1, -1):
        a = ro[i] * _tree_dot(old_stps[i, :n], q[:n])
        al[i] = a
        q[:n] -= a * old_dirs[i, :n]


def lbfgs_forward(old_stps, old_dirs, ro, r, al, num_old, n):
    """core/seis_numerics.py:511-559 (including its i <= num_old bound)."""
    n = int(n)
    for i in range(0, int(num_old) + 1):
        be = ro[i] * _tree_dot(old_dirs[i, :n], r[:n])
        r[:n] += (al[i] - be) * old_stps[i, :n]


KERNELS = {
    "lapg": lapg,
    "update_p": update_p,
    "update_p_diff": update_p_diff,
    "update_p_adjoint": update_p_adjoint,
    "lbfgs_backward": lbfgs_backward,
    "lbfgs_forward": lbfgs_forward,
}
