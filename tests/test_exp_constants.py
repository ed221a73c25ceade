"""The exponential's constants in the device headers equal the ones derived
from exact integer arithmetic by mole_gb300/gen_exp_constants.py: the ln2/64
splits of the FP64 and double-float reductions, 64/ln2 in FP32, the
double-float 1/6, and both 2^(j/64) tables."""
import os
import re
from fractions import Fraction

import numpy as np

from mole_gb300 import gen_exp_constants as G

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "mole_gb300", "csrc")


def _read(name):
    with open(os.path.join(CSRC, name)) as f:
        return f.read()


def _hexf(tok):
    return float.fromhex(tok.rstrip("f"))


def test_exact_arithmetic_basics():
    ln2 = Fraction(G.ln2_fixed(), 1 << G.P)
    assert abs(float(ln2) - np.log(2.0)) < 1e-16
    assert G.exp2_fixed(0) == 1 << G.P and G.exp2_fixed(64) == 2 << G.P
    assert float(Fraction(G.exp2_fixed(32), 1 << G.P)) == np.sqrt(2.0)


def test_fp64_header_constants():
    c = G.constants()
    s = _read("fp64.cuh")
    assert int(re.search(r"kExpL1Int = (0x[0-9A-Fa-f]+)ull", s).group(1), 16) == c["kExpL1Int"]
    assert _hexf(re.search(r"kL2h = (\S+);", s).group(1)) == c["kL2h"]
    assert _hexf(re.search(r"kL2l = (\S+);", s).group(1)) == c["kL2l"]
    inv = re.search(r"__fmul_rn\(xf, ([0-9.]+)f\)\);  // 64 / ln2", s).group(1)
    assert float(np.float32(float(inv))) == c["inv_ln2_64"]
    six = re.search(r"df64\((0x[0-9a-fp.+-]+f), (-?0x[0-9a-fp.+-]+f)\);  // 1/6 \+ r t", s)
    assert (_hexf(six.group(1)), _hexf(six.group(2))) == c["sixth"]


def test_df64_header_constants_and_tables():
    c = G.constants()
    s = _read("df64.cuh")
    assert _hexf(re.search(r"kInv = (\S+);", s).group(1)) == c["inv_ln2_64"]
    assert _hexf(re.search(r"constexpr float kL1 = (\S+);", s).group(1)) == c["df_kL1"]
    assert _hexf(re.search(r"constexpr float kL2 = (\S+);", s).group(1)) == c["df_kL2"]
    assert _hexf(re.search(r"constexpr float kL3 = (\S+);", s).group(1)) == c["df_kL3"]
    tab = s[s.index("kExp2Tab64[64] = {"):]
    tab = tab[:tab.index("};")]
    vals = [float.fromhex(t) for t in re.findall(r"0x[0-9a-f.]+p[+-]\d+", tab)]
    assert vals == c["exp2_tab64"]
    tdf = s[s.index("kExp2TabDF[64][2] = {"):]
    tdf = tdf[:tdf.index("};")]
    pairs = re.findall(r"\{(-?0x[0-9a-f.]+p[+-]\d+)f, (-?0x[0-9a-f.]+p[+-]\d+)f\}", tdf)
    assert [(float.fromhex(a), float.fromhex(b)) for a, b in pairs] == c["exp2_tab_df"]
