"""Build libxara_gpu.so in-tree with nvcc for sm_103a (no CMake)."""
import concurrent.futures as cf
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libxara_gpu.so")
import platform

OBJ = os.path.join(HERE, "_build", platform.machine())
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O2",
                  "--expt-relaxed-constexpr"]


_MACHINES = {"x86_64": 62, "aarch64": 183}


def elf_matches_host(path):
    """True when the ELF file at path was built for this machine."""
    try:
        with open(path, "rb") as f:
            head = f.read(20)
    except OSError:
        return False
    if len(head) < 20 or head[:4] != b"\x7fELF":
        return False
    return int.from_bytes(head[18:20], "little") == _MACHINES.get(platform.machine(), -1)


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)
                  if f.endswith((".cu", ".cpp")))


def _compile(src):
    obj = os.path.join(OBJ, os.path.basename(src) + ".o")
    deps = [src] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith(".h")]
    deps.append(os.path.join(HERE, "..", "include", "xara_gpu.h"))
    if elf_matches_host(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj
    cmd = ["nvcc"] + NVFLAGS + ["-c", src, "-o", obj]
    if src.endswith(".cpp"):
        cmd = ["nvcc", "-x", "cu"] + NVFLAGS + ["-c", src, "-o", obj]
    subprocess.run(cmd, check=True)
    return obj


def build(force=False):
    os.makedirs(OBJ, exist_ok=True)
    srcs = sources()
    if force:
        for f in os.listdir(OBJ):
            os.remove(os.path.join(OBJ, f))
    with cf.ThreadPoolExecutor(max(1, min(len(srcs), os.cpu_count() or 1))) as ex:
        objs = list(ex.map(_compile, srcs))
    if (elf_matches_host(LIB) and
            os.path.getmtime(LIB) >= max(os.path.getmtime(o) for o in objs)):
        return LIB
    tmp = LIB + ".tmp"
    subprocess.run(["nvcc"] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"], check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build())
