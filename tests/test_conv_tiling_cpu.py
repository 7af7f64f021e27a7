"""Index arithmetic of the tcgen05 convolution (csrc/learned.cu), checked on
the CPU.

The kernel stages a 32-channel slab as K-major, no-swizzle core matrices:
8 rows of 16 bytes.  A shared-memory descriptor addresses element (row, k)
at start + (row // 8) * SBO + (k // 8) * LBO + (row % 8) * 16 + (k % 8) * 2.

* A (pixels x channels): the 18 x 10 halo tile of each 8-channel chunk is
  stored as 180 lines of 16 bytes, so LBO = 2880 and SBO = 160.  Tap
  (dy, dx) moves the start by ((1+dy) * 10 + 1+dx) lines, and the K16 step kk
  by 2 * 2880 bytes.
* B (output channels x channels): per tap, [row // 8][k // 8][row % 8], so
  LBO = 128 and SBO = 512.
* TMEM lane m of the accumulator is output pixel (i0 + m // 8, j0 + m % 8).

This test restates the staging and the descriptor offsets.  It checks that
every (M, K) and (N, K) element an MMA addresses is the implicit-GEMM element
x[pixel + (dy, dx)][c0 + k] or w[tap][n][c0 + k].
"""
import numpy as np

TI, TJ, HJ, LINES = 16, 8, 10, 180
LBO_A, SBO_A = LINES * 16, HJ * 16


def _stage_a(i0, j0, H, W, c0, cin):
    """Byte offset -> (i, j, channel) written by the A loader (None = zero)."""
    smem = {}
    for e in range(4 * LINES):
        c, L = divmod(e, LINES)
        hr, hc = divmod(L, HJ)
        i, j, ch = i0 - 1 + hr, j0 - 1 + hc, c0 + c * 8
        ok = 0 <= i < H and 0 <= j < W and ch < cin
        for t in range(8):  # the 16 bytes of one cp.async
            smem[c * LBO_A + L * 16 + 2 * t] = (i, j, ch + t) if ok else None
    return smem


def _stage_b(n0, cout, c0, BN):
    """Byte offset (within one tap's block) -> (co, channel)."""
    smem = {}
    for row in range(BN):
        for c in range(4):
            for t in range(8):
                off = (row >> 3) * 512 + (row & 7) * 16 + c * 128 + 2 * t
                co = n0 + row
                smem[off] = (co, c0 + c * 8 + t) if co < cout else None
    return smem


def _desc_addr(start, lbo, sbo, row, k):
    return start + (row // 8) * sbo + (k // 8) * lbo + (row % 8) * 16 + (k % 8) * 2


def test_a_operand_is_the_shifted_input():
    H, W, cin = 37, 21, 24  # partial tiles, channels beyond cin zero-filled
    for i0, j0 in [(0, 0), (16, 8), (32, 16)]:
        smem = _stage_a(i0, j0, H, W, c0=0, cin=cin)
        for tap in range(9):
            dy, dx = tap // 3 - 1, tap % 3 - 1
            aoff = ((tap // 3) * HJ + (tap % 3)) * 16
            for kk in range(2):
                start = kk * 2 * LBO_A + aoff
                for m in range(128):
                    i, j = i0 + m // TJ, j0 + m % TJ  # TMEM lane m <-> pixel
                    for k in range(16):
                        got = smem[_desc_addr(start, LBO_A, SBO_A, m, k)]
                        ch = kk * 16 + k
                        si, sj = i + dy, j + dx
                        inside = 0 <= si < H and 0 <= sj < W and ch < cin
                        assert got == ((si, sj, ch) if inside else None), (i0, j0, tap, m, k, got)


def test_a_reads_stay_inside_the_slab():
    top = max(_desc_addr(kk * 2 * LBO_A + ((tap // 3) * HJ + tap % 3) * 16, LBO_A, SBO_A, m, k)
              for tap in range(9) for kk in range(2) for m in range(128) for k in range(16))
    assert top + 2 <= 4 * LBO_A  # 11520-byte A slab


def test_b_operand_is_the_weight_tile():
    for BN, cout in [(32, 32), (64, 64), (64, 40), (32, 8)]:
        smem = _stage_b(0, cout, c0=32, BN=BN)
        for kk in range(2):
            for n in range(BN):
                for k in range(16):
                    got = smem[_desc_addr(kk * 256, 128, 512, n, k)]
                    assert got == ((n, 32 + kk * 16 + k) if n < cout else None), (BN, n, k)
