"""Build recipe for the oracle libraries (test infrastructure only).

    python oracle/build_ref.py            # builds oracle/liborc.so and, if possible, oracle/_ref/libref.so

oracle/liborc.so   - the CPU restatement (oracle/mps_oracle.cpp), always built.
oracle/_ref/librefgpu.so, librefgpu_nofma.so - five of the reference's particle kernels
    compiled for sm_103a (oracle/ref_gpu_harness.cu), with and without multiply-add
    contraction: the second baseline and a bit-for-bit check on the GPU.
oracle/_ref/libref.so - the reference solver's own kernel header compiled for the CPU
    by oracle/ref_harness.cpp.  Its sources are decoded copies of four files of the
    reference tree (radix/SPVSOLVER/MultiGPUSolver/{DataType.h, Constant.h,
    Utility_Inline.h, DeviceProcess_Kernel.h}; DataType.h is UTF-16 with a BOM) that
    this script writes to oracle/_ref/src/ when the reference checkout is present
    (at $MPS_REFERENCE_ROOT, by default /root/reference).
    oracle/_ref/ is git-ignored; on a machine without the reference checkout the
    copies already in oracle/_ref/src/ (if any) are compiled, otherwise the reference
    harness is skipped and the pin tests fall back to the committed golden vectors.

Both libraries are compiled with -ffp-contract=off so that the compiler does not fuse
multiply-adds: the oracle and the reference harness then round exactly as their
source text says, on x86-64 and on aarch64 alike.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# checkout of the reference project: MPS_REFERENCE_ROOT, by default /root/reference
REF_ROOT = os.environ.get("MPS_REFERENCE_ROOT", "/root/reference")
REF_TREE = os.path.join(REF_ROOT, "radix", "SPVSOLVER", "MultiGPUSolver")
REF_FILES = ["DataType.h", "Constant.h", "Utility_Inline.h", "DeviceProcess_Kernel.h"]
CXXFLAGS = ["-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared"]


def _decode(src: str, dst: str) -> None:
    raw = open(src, "rb").read()
    if raw[:2] in (b"\xff\xfe", b"\xfe\xff"):
        text = raw.decode("utf-16")
    else:
        text = raw.decode("utf-8", errors="replace")
    with open(dst, "w", encoding="utf-8") as f:
        f.write(text)


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build_oracle(verbose: bool = False) -> str:
    out = os.path.join(HERE, "liborc.so")
    srcs = [os.path.join(HERE, "mps_oracle.cpp"), os.path.join(HERE, "mps_oracle.h")]
    if _stale(out, srcs):
        cmd = ["g++"] + CXXFLAGS + ["-fopenmp", srcs[0], "-o", out]
        if verbose:
            print(" ".join(cmd))
        subprocess.check_call(cmd)
    return out


def build_ref(verbose: bool = False):
    """Returns the path of oracle/_ref/libref.so, or None when no sources exist."""
    ref_dir = os.path.join(HERE, "_ref")
    src_dir = os.path.join(ref_dir, "src")
    if os.path.isdir(REF_TREE):
        os.makedirs(src_dir, exist_ok=True)
        for name in REF_FILES:
            dst = os.path.join(src_dir, name)
            src = os.path.join(REF_TREE, name)
            if _stale(dst, [src]):
                _decode(src, dst)
    if not all(os.path.exists(os.path.join(src_dir, n)) for n in REF_FILES):
        return None
    out = os.path.join(ref_dir, "libref.so")
    harness = os.path.join(HERE, "ref_harness.cpp")
    deps = [harness] + [os.path.join(src_dir, n) for n in REF_FILES]
    if _stale(out, deps):
        cmd = ["g++"] + CXXFLAGS + ["-fopenmp", "-w", "-I" + os.path.join(HERE, "ref_shim"), "-I" + src_dir, harness,
                                    "-o", out]
        if verbose:
            print(" ".join(cmd))
        subprocess.check_call(cmd)
    return out


def _nvcc():
    import shutil
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    return None


def build_ref_gpu(verbose: bool = False):
    """The reference's particle kernels compiled for sm_103a by oracle/ref_gpu_harness.cu:
    oracle/_ref/librefgpu.so (nvcc's default multiply-add contraction, as the reference's
    project builds them) and oracle/_ref/librefgpu_nofma.so (-fmad=false, for bit-for-bit
    comparison).  Returns the two paths, or None when the decoded sources or nvcc are
    missing.  Call build_ref first (it writes the decoded copies)."""
    src_dir = os.path.join(HERE, "_ref", "src")
    nvcc = _nvcc()
    if nvcc is None or not all(os.path.exists(os.path.join(src_dir, n)) for n in REF_FILES):
        return None
    harness = os.path.join(HERE, "ref_gpu_harness.cu")
    deps = [harness] + [os.path.join(src_dir, n) for n in REF_FILES]
    outs = []
    for name, extra in (("librefgpu.so", []), ("librefgpu_nofma.so", ["-fmad=false"])):
        out = os.path.join(HERE, "_ref", name)
        if _stale(out, deps):
            cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-shared",
                   "-Xcompiler", "-fPIC", "-cudart", "static", "-w", "-I" + src_dir] + extra + [harness, "-o", out]
            if verbose:
                print(" ".join(cmd))
            subprocess.check_call(cmd)
        outs.append(out)
    return tuple(outs)


if __name__ == "__main__":
    print(build_oracle(verbose=True))
    print(build_ref(verbose=True))
    print(build_ref_gpu(verbose=True))
    sys.exit(0)
