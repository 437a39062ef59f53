"""The (sin, cos)(2 pi k / 256) table of the light-update kernels (a device constant in
minijclsquant_gb300/csrc/kpm_driven.cu): every entry is the exact value rounded to the
nearest double.  Read from the source and recomputed here in 60-digit arithmetic (CPU)."""
import os
import re

import pytest

from conftest import ROOT

SRC = os.path.join(ROOT, "minijclsquant_gb300", "csrc", "kpm_driven.cu")


def _table():
    text = open(SRC).read()
    body = text[text.index("g_sincos_tab[256] = {"):]
    body = body[: body.index("};")]
    pairs = re.findall(r"\{([^{},]+),\s*([^{},]+)\}", body)
    return [(float.fromhex(a) if "0x" in a else float(a), float.fromhex(b) if "0x" in b else float(b))
            for a, b in pairs]


def test_table_entries_are_correctly_rounded():
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.dps = 60
    tab = _table()
    assert len(tab) == 256
    for k, (s, c) in enumerate(tab):
        x = mpmath.mpf(k) / 128  # 2 pi k / 256 = pi x; sinpi / cospi are exact at multiples of 1/2
        assert s == float(mpmath.sinpi(x)) and c == float(mpmath.cospi(x)), k
    assert tab[0] == (0.0, 1.0) and tab[64] == (1.0, 0.0) and tab[128] == (0.0, -1.0) and tab[192] == (-1.0, 0.0)
