"""Compile check of the reference-side bindings, include/tracetransform_bindings.cpp
(test infrastructure only).

Compiles the file with g++ -fsyntax-only against the reference's own
headers (c++/src/*.hpp of a maleadt/tracetransform checkout, given as the
first argument or $REF, else the recipe's default checkout) on the stand-in
Eigen / Boost headers in oracle/shim/ and the engine's
include/tracetransform.h, with -Werror=missing-declarations: a binding whose
signature drifts from the reference's declaration fails instead of silently
adding an overload.

    python oracle/check_integration.py [REF]     # exit 0: the bindings compile
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
DEFAULT_REF = "/root/reference"  # the checkout this recipe reads when none is given


def main(argv):
    ref = argv[1] if len(argv) > 1 else os.environ.get("REF", DEFAULT_REF)
    src = os.path.join(ref, "c++", "src")
    if not os.path.isdir(src):
        print("no reference checkout at %s" % ref)
        return 2
    cmd = ["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-Wmissing-declarations",
           "-Werror=missing-declarations", "-I", os.path.join(HERE, "shim"), "-I", src,
           "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "include", "tracetransform_bindings.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        print(r.stderr)
    return r.returncode


if __name__ == "__main__":
    sys.exit(main(sys.argv))
