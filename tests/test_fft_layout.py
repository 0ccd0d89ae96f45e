"""Shared-memory layout of the radix line FFT (dlux_gb300/csrc/fft.cu), restated.

`smem_slot` XORs the low nibble of an in-line index with every higher
nibble and with a per-line pattern; `radix_pass` reads the 2^R elements
k0 + m h of each group. For every P the kernel supports (16 ... 8192):
- the map must be a bijection;
- from P = 256 on, the 16 threads of a shared-memory wavefront (8-byte
  words) must hit 16 distinct bank pairs in every radix-16 pass; radix-8
  passes (the schedule below P = 4096) and smaller P may conflict 2-way;
- the scatter of the bit-reversed load may conflict at most 4-way, the
  gathers 2-way.
"""

import pathlib
import re

import pytest

_SRC = (pathlib.Path(__file__).resolve().parents[1] / "dlux_gb300" / "csrc" / "fft.cu").read_text()


def _threshold(pattern):
    m = re.search(pattern, _SRC)
    assert m, f"fft.cu no longer has the form this model restates: {pattern}"
    return int(m.group(1))


# the kernel's own choices, read from its source so that the model follows it
_LPB4_MAX_P = _threshold(r"int lines_per_block\(int P\) \{ return P <= (\d+) \? 4 : 2; \}")
_RADIX16_MIN_P = _threshold(r"int max_radix_log2\(int P\) \{ return P >= (\d+) \? 4 : 3; \}")


def test_model_matches_the_kernel_source():
    assert "(k ^ (((k >> 4) ^ (k >> 8) ^ (k >> 12) ^ g) & 15))" in _SRC
    assert "LPB == 2 ? 9 * li : (LPB == 4 ? 5 * li : li)" in _SRC


def slot(k, li, lpb, P):
    if P < 16:
        return li * P + k
    g = {2: 9 * li, 4: 5 * li}.get(lpb, li)
    return li * P + (k ^ (((k >> 4) ^ (k >> 8) ^ (k >> 12) ^ g) & 15))


def brev(x, bits):
    return int(format(x, f"0{bits}b")[::-1], 2) if bits else 0


def worst_wavefront(slots):
    worst = 1
    for w0 in range(0, len(slots), 16):
        banks = [s % 16 for s in slots[w0:w0 + 16]]
        worst = max(worst, max(banks.count(b) for b in set(banks)))
    return worst


def passes(log2p, rmax):
    out, s = [], 1
    while s <= log2p:
        r = min(rmax, log2p - s + 1)
        out.append((r, s - 1))
        s += r
    return out


def lines_per_block(P):
    return 4 if P <= _LPB4_MAX_P else 2


@pytest.mark.parametrize("log2p", range(4, 14))
def test_slot_map_is_a_bijection_and_passes_are_conflict_free(log2p):
    P = 1 << log2p
    for lpb in (2, 4):
        for li in range(lpb):
            assert sorted(slot(k, li, lpb, P) - li * P for k in range(P)) == list(range(P))
    lpb = lines_per_block(P)
    for rmax in (3, 4):   # both schedules; the kernel uses 4 from P = _RADIX16_MIN_P on
        bound = 1 if (P >= 256 and rmax == 4) else 2
        if rmax == 4 and P >= _RADIX16_MIN_P:
            assert bound == 1   # the kernel's radix-16 sizes are conflict-free
        for R, lh in passes(log2p, rmax):
            gq = log2p - R
            for m in range(1 << R):
                s = []
                for t in range(min(256, lpb << gq)):   # the first warps of a 256-thread block
                    li, i = t >> gq, t & ((1 << gq) - 1)
                    k0 = ((i >> lh) << (lh + R)) + (i & ((1 << lh) - 1))
                    s.append(slot(k0 + m * (1 << lh), li, lpb, P))
                assert worst_wavefront(s) <= bound, (P, rmax, R, lh, m)


@pytest.mark.parametrize("log2p", range(4, 14))
def test_scatter_and_gather_conflicts_are_bounded(log2p):
    P = 1 << log2p
    lpb = lines_per_block(P)
    for line_fast in (True, False):
        for off in (0, 5, P // 3):
            sc, ga = [], []
            for t in range(min(256, lpb * P)):
                li, e = (t % lpb, t // lpb) if line_fast else (t // P, t % P)
                sc.append(slot(brev((e + off) % P, log2p), li, lpb, P))
                ga.append(slot((e + off) % P, li, lpb, P))
            assert worst_wavefront(sc) <= 4 and worst_wavefront(ga) <= 2
