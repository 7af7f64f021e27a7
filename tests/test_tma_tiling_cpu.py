"""Index arithmetic of the TMA-staged matvec (csrc/stencil_tma.cu), checked
on the CPU.

For every tile this restates what reaches shared memory:
  * the TMA box, zero-filled outside the grid:
    - x: rows i0-1 .. i0+16, columns j0-2 .. j0+129;
    - Hz eps: rows i0-2 .. i0+15, columns j0-4 .. j0+127;
  * then the wrap patches of the edge tiles.
It then checks that every neighbour a valid cell reads (x: centre, i±1,
j±1; Hz eps: (i,j), (i-1,j), (i-2,j), (i,j-1), (i,j-2)) is the periodic
neighbour of the grid, and never a zero-filled cell.  The same pass checks
that the box start x coordinate is a multiple of 16 bytes.
"""
import numpy as np
import pytest

TI, TJ = 16, 128


def _x_smem(nx, ny, i0, j0):
    """Global flat index held by each x halo cell (-1 = zero)."""
    rows = np.arange(i0 - 1, i0 + TI + 1)[:, None]
    cols = np.arange(j0 - 2, j0 + TJ + 2)[None, :]
    inside = (rows >= 0) & (rows < nx) & (cols >= 0) & (cols < ny)
    s = np.where(inside, rows * ny + cols, -1)
    q = np.arange(TJ)
    if i0 == 0:
        m = j0 + q < ny
        s[0, q[m] + 2] = (nx - 1) * ny + j0 + q[m]
    if i0 + TI >= nx:
        m = j0 + q < ny
        s[nx - i0 + 1, q[m] + 2] = j0 + q[m]
    r = np.arange(TI)
    if j0 == 0:
        m = i0 + r < nx
        s[r[m] + 1, 1] = (i0 + r[m]) * ny + ny - 1
    if j0 + TJ >= ny:
        m = i0 + r < nx
        s[r[m] + 1, ny - j0 + 2] = (i0 + r[m]) * ny
    return s


def _eps_smem(nx, ny, i0, j0):
    """Global flat index held by each Hz eps box cell (-1 = zero)."""
    rows = np.arange(i0 - 2, i0 + TI)[:, None]
    cols = np.arange(j0 - 4, j0 + TJ)[None, :]
    inside = (rows >= 0) & (rows < nx) & (cols >= 0) & (cols < ny)
    s = np.where(inside, rows * ny + cols, -1)
    if i0 == 0:
        for q in range(2 * TJ):
            r, jq = q // TJ, j0 + q % TJ
            if jq < ny:
                s[r, 4 + q % TJ] = ((nx - 2 + r + nx) % nx) * ny + jq
    if j0 == 0:
        for q in range(2 * TI):
            c, iq = q // TI, i0 + q % TI
            if iq < nx:
                s[2 + q % TI, 2 + c] = iq * ny + (ny - 2 + c)
    return s


@pytest.mark.parametrize("nx,ny", [(2, 4), (16, 8), (17, 12), (33, 256), (40, 132), (64, 260),
                                   (256, 256)])
def test_halo_and_patches_give_periodic_neighbours(nx, ny):
    assert ny % 4 == 0  # the kernel's condition
    for i0 in range(0, nx, TI):
        for j0 in range(0, ny, TJ):
            assert ((j0 - 2) * 8) % 16 == 0 and ((j0 - 4) * 4) % 16 == 0 and (j0 * 4) % 16 == 0
            sx = _x_smem(nx, ny, i0, j0)
            se = _eps_smem(nx, ny, i0, j0)
            for ii in range(TI):
                i = i0 + ii
                if i >= nx:
                    break
                for jj in range(min(TJ, ny - j0)):
                    j = j0 + jj
                    r, c = ii + 1, jj + 2
                    want = {"c": i * ny + j, "m": ((i - 1) % nx) * ny + j, "p": ((i + 1) % nx) * ny + j,
                            "l": i * ny + (j - 1) % ny, "r": i * ny + (j + 1) % ny}
                    got = {"c": sx[r, c], "m": sx[r - 1, c], "p": sx[r + 1, c],
                           "l": sx[r, c - 1], "r": sx[r, c + 1]}
                    assert got == want, (nx, ny, i, j, got, want)
                    er, ec = ii + 2, jj + 4
                    we = [i * ny + j, ((i - 1) % nx) * ny + j, ((i - 2) % nx) * ny + j,
                          i * ny + (j - 1) % ny, i * ny + (j - 2) % ny]
                    ge = [se[er, ec], se[er - 1, ec], se[er - 2, ec], se[er, ec - 1], se[er, ec - 2]]
                    assert ge == we, (nx, ny, i, j, ge, we)
