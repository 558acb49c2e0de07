"""The Butcher tables of spectrum_gb300/csrc/spx_rk_tables.h against the reference's own
common/rk_config.hh: every coefficient of every table bit for bit, compiled from the reference's
header by oracle/ref_glue/rk_dump.cc where the reference sources are present."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "spectrum_gb300", "csrc", "spx_rk_tables.h")
ORACLE = os.path.join(ROOT, "oracle")


def our_tables():
    """{number: (stages, order, adaptive, a, b_lower, v, w)} parsed from the header's text."""
    txt = open(HEADER).read()
    index = [tuple(int(x) for x in m.groups()) for m in
             re.finditer(r"\{(\d+), (\d+), (\d+), (\d+), (\d+)\},", txt)]
    body = txt[txt.index("#define SPX_RK_COEFFS_INIT"):txt.index("static const spx_rk_entry")]
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    vals = [float.fromhex(x) if "x" in x else float(x)
            for x in re.findall(r"-?0x[0-9a-f.]+p[-+]\d+|-?\d+\.\d+", body)]
    out = {}
    for num, s, order, adapt, off in index:
        nlow = s * (s - 1) // 2
        seg = vals[off:off + 3 * s + nlow]
        out[num] = (s, order, adapt, seg[:s], seg[s:s + nlow], seg[s + nlow:2 * s + nlow], seg[2 * s + nlow:])
    return out


def test_header_holds_the_tables_a_context_accepts():
    t = our_tables()
    assert sorted(t) == [n for n in range(33) if n != 30]
    assert t[0][:3] == (1, 1, 0) and t[25][:3] == (4, 4, 0) and t[29][:3] == (7, 5, 1)
    for num, (s, order, adapt, a, low, v, w) in t.items():
        assert len(a) == s and len(v) == s and len(w) == s and len(low) == s * (s - 1) // 2, num
        assert abs(sum(v) - 1.0) < 1e-12, num  # consistent weights
        if adapt:
            assert abs(sum(w) - 1.0) < 1e-12, num


def _have_reference():
    return subprocess.run(["make", "-s", "-C", ORACLE, "has-ref"], stderr=subprocess.DEVNULL).returncode == 0


@pytest.mark.skipif(not _have_reference(), reason="reference sources not present")
def test_tables_equal_the_reference_bit_for_bit():
    subprocess.run(["make", "-s", "-C", ORACLE, "rk-dump"], check=True, stdout=subprocess.DEVNULL)
    ours = our_tables()
    for num, (s, order, adapt, a, low, v, w) in ours.items():
        out = subprocess.run([os.path.join(ORACLE, "_ref", f"rk_dump_{num}")], capture_output=True, text=True,
                             check=True).stdout.split()
        n2, s2, order2, adapt2 = (int(x) for x in out[:4])
        vals = [float.fromhex(x) for x in out[4:]]
        assert (n2, s2, order2, adapt2) == (num, s, order, adapt)
        ra, rb, rv, rw = vals[:s], vals[s:s + s * s], vals[s + s * s:s + s * s + s], vals[s + s * s + s:]
        rlow = [rb[i * s + j] for i in range(s) for j in range(i)]
        for mine, ref in ((a, ra), (low, rlow), (v, rv), (w, rw)):
            assert [x.hex() for x in mine] == [x.hex() for x in ref], num
