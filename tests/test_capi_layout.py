"""The ctypes mirrors of the C ABI's structs (my_swampe_gb300/_lib.py) have
the header's layout: a small C program built with the host compiler prints
sizeof / offsetof of every field of include/swampe_gb300.h's structs, and the
test compares them with ctypes.  No GPU needed."""
import ctypes
import shutil
import subprocess

import pytest

from conftest import ROOT

STRUCTS = {
    "swp_group_state": ("GroupState", ["fourier", "resid", "params", "member", "diag", "hist"]),
    "swp_group_adjoint": ("GroupAdjoint", ["lam", "lam_y", "grad"]),
    "swp_group_tangent": ("GroupTangent", ["fourier", "resid", "dparams", "coef_tangents", "dweights"]),
    "swp_flags": ("Flags", ["scheme", "forcflag", "diffflag", "modalflag", "test", "diagnostics", "blowup",
                            "t_start", "raw_filter"]),
    "swp_emission_cfg": ("EmissionCfg", ["temp_mode", "R_d", "T_ref", "phi_to_T_scale", "Tmin", "model", "nbands",
                                         "wavelengths", "band_weights", "x_clip"]),
}


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    d = tmp_path_factory.mktemp("layout")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "swampe_gb300.h"', "int main(void) {"]
    for cname, (_, fields) in STRUCTS.items():
        lines.append(f'  printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for f in fields:
            lines.append(f'  printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["  return 0;", "}"]
    src = d / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = d / "layout"
    subprocess.run([cc, "-std=c99", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    res = {}
    for line in out.splitlines():
        cname, key, val = line.split()
        res[(cname, key)] = int(val)
    return res


@pytest.mark.parametrize("cname", list(STRUCTS))
def test_ctypes_struct_matches_header(c_layout, cname):
    from my_swampe_gb300 import _lib

    pyname, fields = STRUCTS[cname]
    cls = getattr(_lib, pyname)
    assert [f[0] for f in cls._fields_] == fields, "field order"
    assert ctypes.sizeof(cls) == c_layout[(cname, "sizeof")]
    for f in fields:
        assert getattr(cls, f).offset == c_layout[(cname, f)], f


def test_tangent_rows_match_the_header():
    from my_swampe_gb300 import _lib

    text = (ROOT / "include" / "swampe_gb300.h").read_text()
    assert f"#define SWP_NTANGENT {_lib.NTANGENT}" in text
    assert f"#define SWP_EMISSION_MAX_BANDS {_lib.EMISSION_MAX_BANDS}" in text
