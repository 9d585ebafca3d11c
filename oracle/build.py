"""Builds of the test infrastructure under oracle/ (never imported by the product package).

  build_oracle()          oracle/liboracle.so from the plain-C restatement (gcc, OpenMP when available)
  build_reference(root)   oracle/_ref/libb3ref.so from the reference's own CPU sources under `root`
                          (oracle/build_ref.sh: g++ on the sources where they lie, nothing copied)
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
ORACLE_LIB = HERE / "liboracle.so"
ORACLE_SOURCES = ["b3oracle.c", "b3hull.c"]
ORACLE_HEADERS = ["b3oracle.h"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(map(str, cmd))}\n{r.stdout}\n{r.stderr}")
    return r


def _newer(target: Path, sources) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(s).stat().st_mtime > t for s in sources)


def build_oracle(force: bool = False) -> Path:
    srcs = [HERE / s for s in ORACLE_SOURCES if (HERE / s).exists()]
    deps = srcs + [HERE / h for h in ORACLE_HEADERS]
    if not force and not _newer(ORACLE_LIB, deps):
        return ORACLE_LIB
    tmp = ORACLE_LIB.with_suffix(".so.tmp")
    base = ["gcc", "-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-shared", "-o", str(tmp)] + \
           [str(s) for s in srcs] + ["-lm"]
    try:
        _run(base[:1] + ["-fopenmp"] + base[1:])
    except RuntimeError:
        _run(base)
    os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def build_reference(ref_root: str | None) -> Path | None:
    """oracle/_ref/libb3ref.so from the reference sources under ref_root (None or absent: skipped),
    and oracle/_ref/source_root naming that root."""
    if not ref_root or not Path(ref_root, "src", "Bullet3Common").is_dir():
        return None
    out = HERE / "_ref" / "libb3ref.so"
    out.parent.mkdir(exist_ok=True)
    # where the reference's sources were found (tests that read them look here)
    (HERE / "_ref" / "source_root").write_text(str(Path(ref_root).resolve()))
    if out.exists() and out.stat().st_mtime > (HERE / "ref_shim.cpp").stat().st_mtime:
        return out
    _run(["bash", str(HERE / "build_ref.sh"), ref_root])
    return out


def reference_root() -> Path | None:
    """The reference source root the last build_reference used, when it is still present."""
    p = HERE / "_ref" / "source_root"
    if not p.exists():
        return None
    root = Path(p.read_text().strip())
    return root if (root / "src" / "Bullet3Common").is_dir() else None


if __name__ == "__main__":
    import sys
    print(build_oracle(force=True))
    print(build_reference(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("B3G_REFERENCE_ROOT")))
