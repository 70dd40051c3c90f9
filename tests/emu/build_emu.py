"""TEST INFRASTRUCTURE: builds tests/_build/libffip_emu.so — the engine's host
code (ffip_gb300/csrc/{plan,engine,capi}.cpp) linked with the host emulation
backend (tests/emu/host_backend.cpp) instead of the CUDA kernels."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
CSRC = os.path.join(ROOT, "ffip_gb300", "csrc")
OUT = os.path.join(ROOT, "tests", "_build", "libffip_emu.so")
CLI = os.path.join(ROOT, "tests", "_build", "run_sim_json_emu")


def build() -> str:
    srcs = [os.path.join(CSRC, f) for f in ("plan.cpp", "engine.cpp", "capi.cpp")] + [os.path.join(HERE, "host_backend.cpp")]
    deps = srcs + [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "ffip_gb300.h")]
    if os.path.exists(OUT) and os.path.getmtime(OUT) >= max(os.path.getmtime(d) for d in deps):
        return OUT
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    tmp = OUT + ".tmp%d" % os.getpid()
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-fopenmp", "-I", CSRC, "-I", os.path.join(ROOT, "include"),
                           *srcs, "-o", tmp])
    os.replace(tmp, OUT)
    return OUT


def build_cli() -> str:
    """The run_sim_json driver linked with the emulation library."""
    lib = build()
    src = os.path.join(CSRC, "run_sim_json.cpp")
    if os.path.exists(CLI) and os.path.getmtime(CLI) >= max(os.path.getmtime(src), os.path.getmtime(lib)):
        return CLI
    tmp = CLI + ".tmp%d" % os.getpid()
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-I", CSRC, "-I", os.path.join(ROOT, "include"), src,
                           lib, "-Wl,-rpath," + os.path.dirname(lib), "-o", tmp])
    os.replace(tmp, CLI)
    return CLI


if __name__ == "__main__":
    print(build())
