"""Build the reference's own kernels on the CPU into oracle/_ref/.

Test infrastructure only.  The reference (AnySparse/BMS2, namespace sigmo) is a
header-only SYCL library; this image has no SYCL compiler or runtime.  This
recipe
  1. copies the reference's headers (library/include/*.hpp) from the reference
     tree into oracle/_ref/include/, applying the disclosed patches below —
     each one asserts that the original text is present, so a changed
     reference fails loudly instead of building something else;
  2. compiles oracle/ref/ref_driver.cpp against those headers and the
     host-only SYCL stand-in oracle/ref/sycl/sycl.hpp with g++, into
     oracle/_ref/ref_driver.
Nothing of the reference is committed: oracle/_ref/ is git-ignored.

Patches (nothing else is changed):
  P1 isomorphism.hpp:866 — a line holding only ")" inside
     joinWithPartialMatches: a syntax error for every compiler.  Removed.
  P2 signature.hpp:212, 249, 297, 335 — explicit specialisations of the member
     templates refineAMSignatures / refineCSRSignatures at class scope, which
     g++ rejects.  Each becomes an ordinary member function with a suffixed
     name, and the primary template's declaration becomes a definition that
     calls the suffixed function selected by its Algorithm argument (if
     constexpr).  The function bodies are untouched.

Usage: python oracle/ref/build_ref.py [REFERENCE_ROOT]   (default /root/reference)
"""
from __future__ import annotations

import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ORACLE = HERE.parent
OUT = ORACLE / "_ref"
INC = OUT / "include"
DRIVER = OUT / "ref_driver"
DEFAULT_REF = Path("/root/reference")

HEADERS = ["candidates.hpp", "device.hpp", "gmcr.hpp", "graph.hpp", "io.hpp", "isomorphism.hpp", "pool.hpp",
           "sigmo.hpp", "signature.hpp", "types.hpp", "utils.hpp"]


def _replace_once(text: str, old: str, new: str, what: str) -> str:
    n = text.count(old)
    if n != 1:
        raise RuntimeError(f"patch {what}: expected the original text once, found it {n} times")
    return text.replace(old, new)


def patch_isomorphism(text: str) -> str:
    lines = text.split("\n")
    # line 866 (1-based) holds only ")"
    if lines[865].strip() != ")":
        raise RuntimeError("patch P1: isomorphism.hpp:866 is not the lone ')' this recipe removes")
    del lines[865]
    return "\n".join(lines)


def patch_signature(text: str) -> str:
    for fam, graph in (("refineAMSignatures", "DeviceBatchedAMGraph"), ("refineCSRSignatures", "DeviceBatchedCSRGraph")):
        decl = (f"  template<Algorithm _A = A>\n  utils::BatchedEvent {fam}({graph}& graphs, size_t view_size, "
                f"SignatureScope s);")
        disp = (f"  template<Algorithm _A = A>\n  utils::BatchedEvent {fam}({graph}& graphs, size_t view_size, "
                f"SignatureScope s) {{\n"
                f"    if constexpr (_A == Algorithm::ViewBased) return {fam}__ViewBased(graphs, view_size, s);\n"
                f"    else return {fam}__PowerGraph(graphs, view_size, s);\n  }}")
        text = _replace_once(text, decl, disp, f"P2 {fam} declaration")
        for alg in ("ViewBased", "PowerGraph"):
            spec = f"  template<>\n  utils::BatchedEvent {fam}<Algorithm::{alg}>({graph}& graphs,"
            text = _replace_once(text, spec, f"  utils::BatchedEvent {fam}__{alg}({graph}& graphs,",
                                 f"P2 {fam}<{alg}>")
    return text


def build(ref_root: Path = DEFAULT_REF, force: bool = False) -> Path:
    src = Path(ref_root) / "library" / "include"
    if not src.is_dir():
        raise FileNotFoundError(f"reference headers not found under {src}")
    INC.mkdir(parents=True, exist_ok=True)
    for h in HEADERS:
        text = (src / h).read_text()
        if h == "isomorphism.hpp":
            text = patch_isomorphism(text)
        elif h == "signature.hpp":
            text = patch_signature(text)
        (INC / h).write_text(text)
    (OUT / "PATCHES.txt").write_text(__doc__)
    deps = [HERE / "ref_driver.cpp", HERE / "sycl" / "sycl.hpp"] + [INC / h for h in HEADERS]
    if force or not DRIVER.exists() or any(d.stat().st_mtime > DRIVER.stat().st_mtime for d in deps):
        cxx = shutil.which("g++") or "g++"
        # -O0: the reference reads uninitialised private memory and shifts
        # 64-bit words by more than 63 (its Bitset with global ids); unoptimised
        # code keeps both literal (memory as the stand-in fills it, the
        # hardware shift) instead of leaving them to the optimiser
        cmd = [cxx, "-std=c++20", "-O0", "-w", "-DSIGMO_ALLOCATION=1", "-I", str(HERE), "-I", str(INC),
               str(HERE / "ref_driver.cpp"), "-o", str(DRIVER)]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("reference build failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr[-6000:])
    return DRIVER


if __name__ == "__main__":
    print(build(Path(sys.argv[1]) if len(sys.argv) > 1 else DEFAULT_REF, force="--force" in sys.argv))
