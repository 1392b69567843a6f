"""The C-ABI library loads without a GPU and exports every symbol include/*.h declares."""
import ctypes as C
import re
from pathlib import Path

from mohid_gb300 import _native as N
from oracle import oracle as O

ROOT = Path(__file__).resolve().parent.parent


def _declared():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        txt = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(mohid_[a-z0-9_]+)\s*\(", txt))
    return names


def test_every_declared_symbol_is_exported(built):
    lib = C.CDLL(str(N.lib_path("libmohid_ad.so")))
    declared = _declared()
    assert declared, "no declarations found"
    missing = [n for n in sorted(declared) if not hasattr(lib, n)]
    assert not missing, missing


def test_python_bindings_cover_declarations(built):
    assert _declared() == set(N.AD_SYMBOLS)


def test_params_struct_mirrors_header():
    txt = (ROOT / "include" / "mohid_ad.h").read_text()
    body = txt[txt.index("typedef struct mohid_ad_params {"):txt.index("} mohid_ad_params;")]
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    fields = []
    for line in body.splitlines()[1:]:
        m = re.match(r"\s*(double|int)\s+(.+);", line)
        if m:
            fields += [(m.group(1), n.strip()) for n in m.group(2).split(",")]
    ct = {"double": C.c_double, "int": C.c_int}
    want = [(n, ct[t]) for t, n in fields]
    assert [(f[0], f[1]) for f in N.MohidAdParams._fields_] == want
    assert [(f[0], f[1]) for f in O.Params._fields_] == want


def test_default_params_cpu_callable(built):
    # a pure host function: callable without a GPU
    p = N.MohidAdParams()
    N.ad_lib().mohid_ad_default_params(C.byref(p))
    assert p.AdvMethodH == 1 and p.TVDLimitationH == 4 and p.VolumeRelMax == 1.5
    assert p.ImpExp_AdvV == 1.0 and p.ImpExp_DifV == 1.0 and p.Docycle_method == 1
    assert p.SchmidtBackground_V == 1e-8
    assert N.ad_lib().mohid_ad_version().startswith(b"mohid-gb300")


def _prototypes():
    """{name: parameter count} of every function include/*.h declares."""
    out = {}
    for h in (ROOT / "include").glob("*.h"):
        txt = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"\b(mohid_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;", txt):
            args = " ".join(m.group(2).split())
            out[m.group(1)] = 0 if args in ("", "void") else args.count(",") + 1
    return out


def test_ctypes_signatures_match_the_header():
    # every binding passes as many arguments as its C prototype takes, so a
    # signature change in the header cannot go unnoticed by the Python mirror
    protos = _prototypes()
    assert set(protos) == set(N.AD_SYMBOLS)
    wrong = {n: (protos[n], len(N._AD_SIGS[n][1])) for n in protos if protos[n] != len(N._AD_SIGS[n][1])}
    assert not wrong, wrong
