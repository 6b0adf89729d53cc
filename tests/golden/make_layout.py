"""Records sizeof/offsetof of the interface structs as compiled from the reference's
own DataType.h (decoded copy in oracle/_ref/src, see oracle/build_ref.py) into
tests/golden/layout_reference.txt.

    python tests/golden/make_layout.py

Needs g++ and the reference sources; tests/test_types.py checks include/mps_types.h
(through the ctypes mirror) against the committed file.
"""
import os
import re
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

STRUCTS = ["CParameter", "CTriangleParameters", "CTriangle", "DragParameter", "CDragTriangle", "CParticle",
           "CDistance", "CGridBox", "CCell"]


def field_names():
    src = open(os.path.join(ROOT, "include", "mps_types.h")).read()
    out = {}
    for s in STRUCTS:
        m = re.search(r"typedef struct " + s + r" \{(.*?)\} " + s + ";", src, re.S)
        names = []
        for line in m.group(1).split("\n"):
            line = line.split("/*")[0].strip()
            mm = re.match(r".*?(\w+)(\[\w+\])?;", line)
            if mm:
                names.append(mm.group(1))
        out[s] = names
    return out


def main():
    import build_ref
    build_ref.build_ref()
    src_dir = os.path.join(ROOT, "oracle", "_ref", "src")
    if not os.path.exists(os.path.join(src_dir, "DataType.h")):
        raise SystemExit("reference sources not available")
    fields = field_names()
    with tempfile.TemporaryDirectory(dir=os.path.join(ROOT, "_build") if os.path.isdir(os.path.join(ROOT, "_build"))
                                     else None) as td:
        cpp = os.path.join(td, "probe.cpp")
        with open(cpp, "w") as f:
            f.write('#include <cstdio>\n#include <cstddef>\n#include "cuda_runtime.h"\n#define __device__\n'
                    '#define __host__\n#define __inline__ inline\n#include "DataType.h"\nint main(){\n')
            for s in STRUCTS:
                f.write(f'printf("{s} %zu\\n", sizeof({s}));\n')
                for fl in fields[s]:
                    f.write(f'printf("{s}.{fl} %zu\\n", offsetof({s},{fl}));\n')
            f.write("}\n")
        exe = os.path.join(td, "probe")
        subprocess.check_call(["g++", "-w", "-I" + os.path.join(ROOT, "oracle", "ref_shim"), "-I" + src_dir, cpp,
                               "-o", exe])
        txt = subprocess.check_output([exe]).decode()
    with open(os.path.join(HERE, "layout_reference.txt"), "w") as f:
        f.write(txt)
    print("written", len(txt.splitlines()), "lines")


if __name__ == "__main__":
    main()
