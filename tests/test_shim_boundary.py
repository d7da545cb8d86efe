"""The Fortran shim is a drop-in for the reference's driver: every name that
app/main.F90 imports from a module the shim replaces is public in the shim's
module of the same name, and every replaced subroutine keeps the reference's
number of dummy arguments.

The imports and the reference's signatures are a committed fixture
(tests/golden/main_f90_imports.json, written by
tests/golden/make_main_imports.py from the reference's sources); when the
reference's sources are present the fixture is also checked against them."""
import json
import re
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
SHIM = ROOT / "bio-cfd_gb300" / "fortran" / "biocfd_gb300_shim.f90"
FIXTURE = ROOT / "tests" / "golden" / "main_f90_imports.json"

sys.path.insert(0, str(ROOT / "tests" / "golden"))
import make_main_imports  # noqa: E402


def _join_continuations(text: str):
    out, cur = [], ""
    for ln in text.splitlines():
        code = ln.split("!", 1)[0].rstrip()
        if cur:
            code = code.lstrip()
            if code.startswith("&"):
                code = code[1:]
            cur += " " + code
        else:
            cur = code
        if cur.endswith("&"):
            cur = cur[:-1]
            continue
        out.append(cur)
        cur = ""
    return out


def shim_modules():
    """module -> {"public": set of names, "subs": {name: [dummy args]}}."""
    mods, cur = {}, None
    for st in _join_continuations(SHIM.read_text()):
        m = re.match(r"^\s*module\s+(\w+)\s*$", st, re.I)
        if m:
            cur = m.group(1).lower()
            mods[cur] = {"public": set(), "subs": {}, "private": False}
            continue
        if re.match(r"^\s*end\s+module", st, re.I):
            cur = None
            continue
        if cur is None:
            continue
        if re.match(r"^\s*private\s*$", st, re.I):
            mods[cur]["private"] = True
        m = re.match(r"^\s*public\s*::(.*)$", st, re.I)
        if m:
            mods[cur]["public"].update(n.strip().lower() for n in m.group(1).split(",") if n.strip())
        m = re.match(r"^\s*subroutine\s+(\w+)\s*(?:\(([^)]*)\))?", st, re.I)
        if m:
            args = [a.strip().lower() for a in (m.group(2) or "").split(",") if a.strip()]
            mods[cur]["subs"][m.group(1).lower()] = args
    return mods


def test_fixture_matches_reference_sources():
    ref = make_main_imports.REFERENCE
    if not (ref / "app" / "main.F90").exists():
        pytest.skip("reference sources not present (the committed fixture stands)")
    fx = json.loads(FIXTURE.read_text())
    assert fx["use_only"] == make_main_imports.parse_use_lists((ref / "app" / "main.F90").read_text())


def test_every_import_of_main_is_public_in_the_shim():
    fx = json.loads(FIXTURE.read_text())
    mods = shim_modules()
    replaced = [m for m in fx["use_only"] if m in mods]
    # the shim replaces exactly these modules of the reference
    assert sorted(replaced) == ["biocfd_boundary_conditions", "biocfd_coefficient_matrix", "biocfd_forcing",
                                "biocfd_navier_stokes", "biocfd_pcor_vcor", "biocfd_search"], replaced
    missing = []
    for mod in replaced:
        info = mods[mod]
        for name in fx["use_only"][mod]:
            visible = name in info["public"] or (not info["private"] and name in info["subs"])
            if not visible or name not in info["subs"]:
                missing.append(f"{mod}::{name}")
    assert not missing, f"names app/main.F90 imports that the shim lacks: {missing}"


def test_replaced_routines_keep_the_reference_arguments():
    fx = json.loads(FIXTURE.read_text())
    mods = shim_modules()
    bad = []
    for mod, names in fx["use_only"].items():
        if mod not in mods:
            continue
        for name in names:
            ref = fx["signatures"].get(name)
            got = mods[mod]["subs"].get(name)
            if ref is None or got is None:
                continue
            if len(ref["args"]) != len(got):
                bad.append(f"{name}: reference {ref['file']} {ref['args']} vs shim {got}")
    assert not bad, bad
