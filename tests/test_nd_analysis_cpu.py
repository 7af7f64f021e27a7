"""Symbolic analysis of the direct preconditioner, checked on the CPU.

`cev_nd_analyse` runs the nested-dissection analysis of csrc/nd.cu (tree,
front sizes, original-entry descriptors, factor layout) without any CUDA
call.  Its counts are compared here with an independent Python restatement
of the same ordering: a box splits its longer side at the midpoint by a
one-cell separator line, boxes with both sides <= 4 are leaves, a node's
interior I is its separator (or leaf box) and its boundary B the one-cell
frame around the box inside the grid.  Every cell must be eliminated exactly
once.  The factor stores [G | H] (nI x f) and -K (nB x nI) per node; the
Gauss-Jordan work is sum nI f^2 complex multiply-adds.
"""
import ctypes as C

import pytest

LEAF = 4


def _tree(nx, ny):
    nodes = []  # (depth, interior cells, boundary cells)
    stack = [(0, nx, 0, ny, 0)]
    while stack:
        x0, x1, y0, y1, d = stack.pop()
        if x1 <= x0 or y1 <= y0:
            continue
        w, h = x1 - x0, y1 - y0
        if w <= LEAF and h <= LEAF:
            interior = [i * ny + j for i in range(x0, x1) for j in range(y0, y1)]
        elif w >= h:
            xs = x0 + w // 2
            interior = [xs * ny + j for j in range(y0, y1)]
            stack += [(xs + 1, x1, y0, y1, d + 1), (x0, xs, y0, y1, d + 1)]
        else:
            ys = y0 + h // 2
            interior = [i * ny + ys for i in range(x0, x1)]
            stack += [(x0, x1, ys + 1, y1, d + 1), (x0, x1, y0, ys, d + 1)]
        frame = []
        if x0 > 0:
            frame += [(x0 - 1) * ny + j for j in range(y0, y1)]
        if x1 < nx:
            frame += [x1 * ny + j for j in range(y0, y1)]
        if y0 > 0:
            frame += [i * ny + y0 - 1 for i in range(x0, x1)]
        if y1 < ny:
            frame += [i * ny + y1 for i in range(x0, x1)]
        nodes.append((d, interior, frame))
    return nodes


def _counts(nx, ny):
    nodes = _tree(nx, ny)
    elems = cmacs = desc = 0
    seen = [0] * (nx * ny)
    for _, interior, frame in nodes:
        nI, nB = len(interior), len(frame)
        f = nI + nB
        elems += nI * f + nB * nI
        cmacs += nI * f * f
        pos = {c: q for q, c in enumerate(interior + frame)}
        for q, cell in enumerate(interior + frame):
            i, j = divmod(cell, ny)
            dirs = ((0, 0), (-1, 0), (1, 0), (0, -1), (0, 1)) if q < nI else \
                ((-1, 0), (1, 0), (0, -1), (0, 1))
            for di, dj in dirs:
                ii, jj = i + di, j + dj
                if not (0 <= ii < nx and 0 <= jj < ny):
                    continue  # no periodic wrap in the factorisation
                p = pos.get(ii * ny + jj)
                if p is not None and (q < nI or p < nI):
                    desc += 1
        for c in interior:
            seen[c] += 1
    depths = 1 + max(d for d, _, _ in nodes)
    return len(nodes), depths, elems, cmacs, desc, seen


@pytest.fixture(scope="module")
def lib():
    from ceviche_gb300 import _lib
    return _lib.load()


@pytest.mark.parametrize("shape", [(2, 2), (7, 5), (13, 11), (40, 36), (97, 80), (64, 200),
                                   (200, 64), (131, 77)])
def test_analysis_matches_restatement(lib, shape):
    nx, ny = shape
    nn, fe, nd = C.c_size_t(), C.c_size_t(), C.c_size_t()
    d, fl, cov = C.c_int(), C.c_double(), (C.c_longlong * 2)()
    assert lib.cev_nd_analyse(nx, ny, C.byref(nn), C.byref(d), C.byref(fe), C.byref(fl),
                              C.byref(nd), cov) == 0
    n_nodes, depths, elems, cmacs, desc, seen = _counts(nx, ny)
    assert all(s == 1 for s in seen)  # the restatement eliminates every cell once
    assert (cov[0], cov[1]) == (0, 0)  # and so does the library
    assert nn.value == n_nodes
    assert d.value == depths
    assert fe.value == elems
    assert fl.value == float(cmacs)
    assert nd.value == desc


def test_analysis_rejects_bad_grids(lib):
    nn = C.c_size_t()
    assert lib.cev_nd_analyse(1, 50, C.byref(nn), None, None, None, None, None) < 0
    assert lib.cev_nd_analyse(50, 1, C.byref(nn), None, None, None, None, None) < 0
