"""Writes main_f90_imports.json: for every `use <module>, only: ...` statement
of the reference's driver (app/main.F90, the caller the Fortran shim must
relink against), the module name and the names it imports, lower-cased.

Run in a checkout that has the reference at REF (default: $BIOCFD_REFERENCE,
else /root/reference):
    python tests/golden/make_main_imports.py [REF]
"""
from __future__ import annotations

import json
import os
import re
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REFERENCE = Path(os.environ.get("BIOCFD_REFERENCE", "/root/reference"))


def parse_use_lists(text: str) -> dict:
    """module -> sorted imported names, over every `use m, only: ...` statement
    (free-form continuation lines joined; preprocessor lines kept, so both
    branches of an #if contribute)."""
    lines = text.splitlines()
    joined, cur = [], ""
    for ln in lines:
        code = ln.split("!", 1)[0].rstrip()
        if code.lstrip().startswith("#"):
            continue
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
        joined.append(cur)
        cur = ""
    out: dict = {}
    pat = re.compile(r"^\s*use\s*(?:,\s*intrinsic\s*)?(?:::)?\s*(\w+)\s*,\s*only\s*:(.*)$", re.I)
    for st in joined:
        m = pat.match(st)
        if not m:
            continue
        mod = m.group(1).lower()
        names = [n.strip().lower() for n in m.group(2).split(",") if n.strip()]
        names = [n.split("=>")[0].strip() for n in names]
        out.setdefault(mod, set()).update(names)
    return {k: sorted(v) for k, v in sorted(out.items())}


def subroutine_signatures(text: str) -> dict:
    """name -> dummy argument names of every SUBROUTINE statement (lower-cased)."""
    out = {}
    pat = re.compile(r"^\s*(?:(?:pure|elemental|recursive|module)\s+)*subroutine\s+(\w+)\s*(?:\(([^)]*)\))?",
                     re.I | re.M)
    for m in pat.finditer(text):
        args = [a.strip().lower() for a in (m.group(2) or "").replace("&", " ").split(",") if a.strip()]
        out[m.group(1).lower()] = args
    return out


def main():
    ref = Path(sys.argv[1]) if len(sys.argv) > 1 else REFERENCE
    src = ref / "app" / "main.F90"
    uses = parse_use_lists(src.read_text())
    sigs = {}
    for f in sorted((ref / "src").glob("*.[fF]90")):
        for name, args in subroutine_signatures(f.read_text(errors="replace")).items():
            sigs.setdefault(name, {"file": f"src/{f.name}", "args": args})
    imported = {n for names in uses.values() for n in names}
    d = {"source": "app/main.F90", "use_only": uses,
         "signatures": {n: sigs[n] for n in sorted(imported) if n in sigs}}
    (HERE / "main_f90_imports.json").write_text(json.dumps(d, indent=1) + "\n")
    print(f"wrote {HERE / 'main_f90_imports.json'}: {sum(len(v) for v in d['use_only'].values())} names")


if __name__ == "__main__":
    main()
