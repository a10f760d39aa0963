"""The oracle's assemble_matrix / assemble_vector (core.jl:164-225 with the
built-in functions): consistency with its own sums and the matrices'
structure (CPU only)."""
import numpy as np
import pytest

from sphgpu import geometry as G


def setup(oracle_mod, dim=2, dr=0.05, seed=1):
    c = G.dam_break(dim, dr)
    o = oracle_mod.from_case(c)
    rng = np.random.default_rng(seed)
    v = rng.normal(0.0, 0.1, c.x.shape)
    if dim == 2:
        v[:, 2] = 0.0
    o.set_state(v=v)
    o.create_cell_list()
    return c, o


def rows(I, n):
    starts = np.searchsorted(I, np.arange(n + 1))
    return starts


def test_kernel_matrix_rows_are_kernel_sums(oracle_mod):
    c, o = setup(oracle_mod)
    I, J, V = o.assemble_matrix(oracle_mod.MAT_KERNEL)
    assert np.all(np.diff(I) >= 0)  # rows in order
    st = rows(I, c.n)
    sums = o.sum_particles(oracle_mod.SUM_KERNEL, np.arange(c.n))
    for p in range(c.n):
        acc = 0.0
        for v in V[st[p]:st[p + 1]]:
            acc = acc + v           # the push order is the sum's order
        assert acc == sums[p]
    # one diagonal entry per row, W(0)
    diag = V[I == J]
    assert diag.size == c.n and np.all(diag == diag[0])


def test_projection_matrix_structure(oracle_mod):
    import scipy.sparse as sp
    c, o = setup(oracle_mod)
    I, J, V = o.assemble_matrix(oracle_mod.MAT_PROJECTION, 10.0)
    A = sp.coo_matrix((V, (I, J)), shape=(c.n, c.n)).tocsr()
    off = A - sp.diags(A.diagonal())
    assert abs(off - off.T).max() == 0.0               # symmetric off-diagonal
    assert (off.data < 0).all()                        # rDW < 0 inside the support
    # diagonal = h^2 L = -(row sum of the off-diagonal), plus the penalty
    rs = -np.asarray(off.sum(axis=1)).ravel()
    wall = c.type == G.WALL
    assert np.allclose(A.diagonal()[wall], rs[wall], rtol=1e-12, atol=0)
    assert (A.diagonal()[~wall] >= rs[~wall] * (1 - 1e-12)).all()
    # positive definite: the penalty rows pin the free surface
    x = np.linalg.solve(A.toarray(), np.ones(c.n))
    assert np.isfinite(x).all()


def test_projection_vector(oracle_mod):
    c, o = setup(oracle_mod)
    b = o.assemble_vector(oracle_mod.VEC_PROJECTION)
    assert b.shape == (c.n,) and np.isfinite(b).all() and np.abs(b).max() > 0
