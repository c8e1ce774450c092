"""The colouring of the multicolour SOR (laboetie_gb300/csrc/pnp.cu:k_sor_color_gen) is proper
on every box shape: no D3Q19 link joins two different nodes of one colour, so a colour's nodes
can be updated in place at once.  Host-side restatement of the kernel's rule; no GPU needed."""
import numpy as np
import pytest


def _colour_py(x, y, z, L):
    """The colour rule of pnp.cu:k_sor_color_gen (ring colours combined per axis pair)."""
    def ring(v, n):
        return 0 if n == 1 else (v & 1 if n % 2 == 0 else (2 if v == n - 1 else v & 1))
    k = [1 if n == 1 else (2 if n % 2 == 0 else 3) for n in L]
    ka, kb = max(k[0], k[2]), max(k[1], k[2])
    gx, gy, gz = ring(x, L[0]), ring(y, L[1]), ring(z, L[2])
    return (gx + gz) % ka + ka * ((gy + gz) % kb), ka * kb


@pytest.mark.parametrize("L", [(1, 1, 64), (1, 1, 63), (1, 1, 2), (9, 9, 9), (9, 9, 4), (7, 8, 5),
                               (2, 3, 5), (1, 5, 7), (48, 48, 48), (3, 3, 3)])
def test_multicolour_rule_is_a_proper_colouring(L):
    """No D3Q19 link joins two different nodes of one colour (a link back to the node itself,
    along a one-wide axis, is not a conflict: the update reads the node's own old value)."""
    from oracle import np_oracle as npo

    lx, ly, lz = L
    col = np.zeros((lz, ly, lx), dtype=int)
    for z in range(lz):
        for y in range(ly):
            for x in range(lx):
                col[z, y, x], n = _colour_py(x, y, z, L)
    assert n <= 9
    for c in npo.C[1:]:
        other = np.roll(col, shift=(-int(c[2]), -int(c[1]), -int(c[0])), axis=(0, 1, 2))
        if all(L[d] == 1 or c[d] == 0 for d in range(3)):
            continue   # the link returns to the node itself
        assert not np.any(other == col), (L, c)
