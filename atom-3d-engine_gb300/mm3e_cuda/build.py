"""Build libmm3e_cuda.so in-tree (sm_103a only).

Device code is compiled by nvcc for `-gencode arch=compute_103a,code=sm_103a` (no fast-math:
the render path needs IEEE division/sqrt and the accurate transcendentals). Host code that
reproduces Rust binary32 arithmetic (scene lowering, camera/rotation helpers) is compiled
with `-ffp-contract=off`. The CUDA runtime is linked statically so the library has no
runtime dependency beyond the driver.
"""
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(ROOT, "csrc")
OUT_DIR = os.path.join(PKG, "_lib")
OBJ_DIR = os.path.join(PKG, "_build")
LIB = os.path.join(OUT_DIR, "libmm3e_cuda.so")
INCLUDE = os.path.join(os.path.dirname(ROOT), "include")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
GENCODE = "arch=compute_103a,code=sm_103a"

CU_SOURCES = ["wavefront.cu", "noalloc.cu", "mesh_bake.cu", "reproject.cu"]
CPP_SOURCES = ["lower.cpp", "capi.cpp", "engine.cpp", "batch.cpp", "mesh.cpp", "server.cpp", "spec.cpp", "spec_gen.cpp", "scene_io.cpp"]
HEADERS = ["tape.h", "lower.h", "kernels.h", "device_math.cuh", "noalloc.h", "engine.h", "capi_internal.h", "batch.h", "mesh.h", "server.h", "march_kernels.cuh", "shade_kernels.cuh", "post_kernels.cuh", "reproject_kernels.cuh", "spec.h"]


def _cudart_dir():
    for cand in (os.path.join(CUDA_HOME, "lib64"), os.path.join(CUDA_HOME, "targets", "sbsa-linux", "lib"),
                 os.path.join(CUDA_HOME, "targets", "x86_64-linux", "lib")):
        if os.path.exists(os.path.join(cand, "libcudart_static.a")):
            return cand
    raise RuntimeError("libcudart_static.a not found under " + CUDA_HOME)


def _deps():
    files = [os.path.join(CSRC, f) for f in CU_SOURCES + CPP_SOURCES + HEADERS]
    files.append(os.path.join(INCLUDE, "mm3e_cuda.h"))
    files.append(os.path.abspath(__file__))
    return files


def stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(f) > t for f in _deps())


# Device sources compiled again at run time by NVRTC for scene-specialised programs.
EMBEDDED = ["tape.h", "device_math.cuh", "kernels.h", "march_kernels.cuh"]


def write_embedded(path):
    """C++ include with the EMBEDDED sources as null-terminated arrays of string-literal chunks."""
    out = ["// generated by mm3e_cuda/build.py from csrc/: device sources for NVRTC", "namespace mm3e {"]
    for name in EMBEDDED:
        with open(os.path.join(CSRC, name)) as f:
            src = f.read()
        ident = "embed_" + name.replace(".", "_")
        out.append(f"static const char* const {ident}[] = {{")
        for i in range(0, len(src), 16000):
            out.append('R"MM3E_EMBED(' + src[i:i + 16000] + ')MM3E_EMBED",')
        out.append("nullptr};")
    out.append("}  // namespace mm3e")
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")


def build(force=False, verbose=False, extra_nvcc=()):
    """Compile (in parallel) and link the library if any input changed. Returns the .so path."""
    if not force and not stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    write_embedded(os.path.join(OBJ_DIR, "embedded_sources.inc"))
    jobs = []
    objs = []
    for src in CU_SOURCES:
        obj = os.path.join(OBJ_DIR, src + ".o")
        # --fmad=false: no multiply-add contraction, so binary32 results follow the reference's
        # (Rust never contracts); hit points then agree bit for bit and the reference's
        # hash-of-position shadow jitter and checker tiles are reproduced.
        cmd = [NVCC, "-gencode", GENCODE, "-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC",
               "-Xptxas", "-v", "-I", INCLUDE, "-c", os.path.join(CSRC, src), "-o", obj, *extra_nvcc]
        jobs.append((cmd, obj))
        objs.append(obj)
    for src in CPP_SOURCES:
        obj = os.path.join(OBJ_DIR, src + ".o")
        cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall",
               "-I", os.path.join(CUDA_HOME, "include"), "-I", INCLUDE, "-I", OBJ_DIR, "-c", os.path.join(CSRC, src),
               "-o", obj]
        jobs.append((cmd, obj))
        objs.append(obj)
    procs = []
    for cmd, obj in jobs:
        if verbose:
            print(" ".join(cmd))
        procs.append((subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT), cmd, obj))
    logs = []
    for p, cmd, obj in procs:
        out, _ = p.communicate()
        text = out.decode(errors="replace")
        logs.append(text)
        if p.returncode != 0:
            sys.stderr.write(text)
            raise RuntimeError("compile failed: " + " ".join(cmd))
    with open(os.path.join(OBJ_DIR, "ptxas.log"), "w") as f:
        f.write("\n".join(logs))
    link = ["g++", "-shared", "-o", LIB + ".tmp", *objs, "-L" + _cudart_dir(), "-lcudart_static", "-lrt", "-ldl",
            "-lpthread"]
    if verbose:
        print(" ".join(link))
    subprocess.check_call(link)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
