"""Compile check of the reference-side bindings in INTEGRATION.md (test
infrastructure only).

Extracts every ```cpp block of INTEGRATION.md and compiles them, with
g++ -fsyntax-only, against the reference's own headers (c++/src/*.hpp of a
maleadt/tracetransform checkout, given as REF or the first argument; by
default /root/reference) on the stand-in Eigen / Boost headers in
oracle/shim/ and the engine's include/tracetransform.h.  Blocks that define
functions are compiled as they are, with -Werror=missing-declarations, so a
binding whose signature drifts from the reference's declaration fails
instead of silently adding an overload; statement fragments are wrapped in
a function whose parameters declare the names they use.

    python oracle/check_integration.py [REF]     # exit 0: every block compiles
"""
import os
import re
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

# Parameters that declare the free names of the statement fragments.
FRAGMENT_PARAMS = {
    "tt_transform(": "const Eigen::MatrixXf &image, unsigned angle_stepsize, "
                     "std::vector<int32_t> ids, int nT, std::vector<tt_pfunctional> pf, "
                     "int nP, int A",
    "tt_transform_batch(": "const float *images, const int64_t *offsets, const int32_t *rows, "
                           "const int32_t *cols, const int32_t *angle_steps, int n_images, "
                           "const int32_t *ids, int nT, const tt_pfunctional *pf, int nP, "
                           "float *circus, float *signatures",
}

PRELUDE = """#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <vector>
#include "sinogram.hpp"
#include "circus.hpp"
#include "auxiliary.hpp"
#include "tracetransform.h"
"""


def blocks(text):
    return re.findall(r"```cpp\n(.*?)```", text, re.S)


def translation_unit(text):
    parts, frag = [PRELUDE], 0
    for b in blocks(text):
        body = b.replace('#include "tracetransform.h"\n', "")
        if re.search(r"^\}\s*$", body, re.M):  # a closing brace at column 0: definitions
            parts.append(body)
            continue
        params = next((p for key, p in FRAGMENT_PARAMS.items() if key in body), None)
        if params is None:
            raise ValueError("no parameter list for fragment:\n" + body)
        parts.append("[[maybe_unused]] static void fragment_%d(%s) {\n%s}\n" % (frag, params, body))
        frag += 1
    return "\n".join(parts)


def main(argv):
    ref = argv[1] if len(argv) > 1 else os.environ.get("REF", "/root/reference")
    src = os.path.join(ref, "c++", "src")
    if not os.path.isdir(src):
        print("no reference checkout at %s" % ref)
        return 2
    tu = translation_unit(open(os.path.join(ROOT, "INTEGRATION.md")).read())
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "bindings.cpp")
        with open(path, "w") as f:
            f.write(tu)
        cmd = ["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-Wmissing-declarations",
               "-Werror=missing-declarations", "-I", os.path.join(HERE, "shim"), "-I", src,
               "-I", os.path.join(ROOT, "include"), path]
        r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        print(r.stderr)
    return r.returncode


if __name__ == "__main__":
    sys.exit(main(sys.argv))
