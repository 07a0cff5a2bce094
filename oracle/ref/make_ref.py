"""Build the parity reference: WaterCube's own GLSL compute shaders compiled as C++.

TEST INFRASTRUCTURE ONLY. This recipe reads the reference's shader sources where they lie
($WC_REFERENCE_ROOT, else a checkout named `reference` beside the repository), removes the three GLSL-only constructs that
C++ cannot parse, and compiles each shader unchanged otherwise against oracle/ref/glsl_compat.h:

  * the `#version` line;
  * `layout(local_size_x = ...) in;` (its local size is kept for the dispatch loop);
  * SSBO blocks `layout(std430, binding = k) <qualifiers> buffer Name { T items[]; };`,
    which become a global `T* items;` that the driver binds;
  and `uniform` becomes a plain global.

Everything goes to oracle/_ref/ (git-ignored): gen/<shader>.cpp, the objects and
libwcref.so. The reference host code (Cinder, Windows.h) is not built; oracle/ref/ref_driver.cpp
replays its dispatch sequence. Where the reference checkout is absent (the GPU machine) but
oracle/_ref/gen/ travelled with the repository, the library is rebuilt from gen/ alone.

Usage: python oracle/ref/make_ref.py [--force]
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
OUT = REPO / "oracle" / "_ref"
GEN = OUT / "gen"
LIB = OUT / "libwcref.so"

# (symbol prefix, path under the reference checkout)
SHADERS = [
    ("count", "assets/sort/count.comp"),
    ("linearScan", "assets/sort/linearScan.comp"),
    ("reorder", "assets/sort/reorder.comp"),
    ("sort", "assets/sort/sort.comp"),
    ("density", "assets/fluid/density.comp"),
    ("update", "assets/fluid/update.comp"),
]

CXXFLAGS = ["-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-std=c++17", "-w"]

_BLOCK = re.compile(
    r"layout\s*\([^)]*\)\s*((?:\w+\s+)*?)buffer\s+(\w+)\s*\{\s*(\w+)\s+(\w+)\s*\[\s*\]\s*;\s*\}\s*;",
    re.S,
)
_LOCAL = re.compile(r"layout\s*\(\s*local_size_x\s*=\s*(\d+)[^)]*\)\s*in\s*;")
_UNIFORM = re.compile(r"^\s*uniform\s+(\w+)\s+(\w+)\s*;", re.M)


def reference_root() -> Path | None:
    """$WC_REFERENCE_ROOT when set, else a WaterCube checkout named `reference` beside this
    repository's directory; None when neither holds the shaders."""
    env = os.environ.get("WC_REFERENCE_ROOT")
    root = Path(env) if env else Path(__file__).resolve().parents[3] / "reference"
    return root if (root / "assets" / "sort" / "count.comp").is_file() else None


def translate(name: str, src: str, origin: str) -> str:
    """GLSL compute shader text -> one C++ translation unit with C-callable glue."""
    src = re.sub(r"^\s*#version[^\n]*\n", "", src, count=1, flags=re.M)
    m = _LOCAL.search(src)
    if not m:
        raise ValueError(f"{origin}: no local_size_x layout")
    local = int(m.group(1))
    src = _LOCAL.sub("", src)
    buffers = []

    def repl(mb: re.Match) -> str:
        elem, var = mb.group(3), mb.group(4)
        buffers.append((elem, var))
        return f"{elem}* {var} = nullptr;"

    src = _BLOCK.sub(repl, src)
    if re.search(r"\bbuffer\b", src):
        raise ValueError(f"{origin}: unparsed buffer block")
    uniforms = _UNIFORM.findall(src)

    ns = f"wcref_{name}"
    glue = [f"extern \"C\" int {ns}_set_buffer(const char* n, void* p) {{"]
    for elem, var in buffers:
        glue.append(f"  if (__builtin_strcmp(n, \"{var}\") == 0) {{ {ns}::{var} = ({ns}::{elem}*)p; return 0; }}")
    glue.append("  return -1;\n}")
    glue.append(f"extern \"C\" int {ns}_set_float(const char* n, const float* v, int k) {{")
    for ty, var in uniforms:
        if ty == "float":
            glue.append(f"  if (k == 1 && __builtin_strcmp(n, \"{var}\") == 0) {{ {ns}::{var} = v[0]; return 0; }}")
        elif ty == "vec3":
            glue.append(
                f"  if (k == 3 && __builtin_strcmp(n, \"{var}\") == 0) "
                f"{{ {ns}::{var} = glsl::vec3(v[0], v[1], v[2]); return 0; }}"
            )
    glue.append("  return -1;\n}")
    glue.append(f"extern \"C\" int {ns}_set_int(const char* n, int v) {{")
    for ty, var in uniforms:
        if ty in ("int", "uint"):
            glue.append(f"  if (__builtin_strcmp(n, \"{var}\") == 0) {{ {ns}::{var} = v; return 0; }}")
    glue.append("  return -1;\n}")
    glue.append(f"extern \"C\" unsigned {ns}_local_size(void) {{ return {local}u; }}")
    glue.append(
        f"extern \"C\" void {ns}_dispatch(unsigned groups, int threads) {{\n"
        f"  const long long total = (long long)groups * {local};\n"
        f"  #pragma omp parallel for schedule(static) num_threads(threads > 0 ? threads : 1)\n"
        f"  for (long long id = 0; id < total; ++id) {{\n"
        f"    gl_GlobalInvocationID = glsl::uvec3((unsigned)id, 0u, 0u);\n"
        f"    {ns}::main();\n"
        f"  }}\n}}"
    )
    return (
        f"// Generated by oracle/ref/make_ref.py from {origin}. Do not edit; not committed.\n"
        f"#include \"glsl_compat.h\"\n"
        f"#define uniform\n"
        f"namespace {ns} {{\nusing namespace glsl;\n{src}\n}}  // namespace {ns}\n"
        f"#undef uniform\n" + "\n".join(glue) + "\n"
    )


def generate(root: Path) -> None:
    GEN.mkdir(parents=True, exist_ok=True)
    for name, rel in SHADERS:
        text = (root / rel).read_text()
        (GEN / f"{name}.cpp").write_text(translate(name, text, rel))


def compile_lib() -> Path:
    OUT.mkdir(parents=True, exist_ok=True)
    jobs = []
    for name, _ in SHADERS:
        jobs.append((GEN / f"{name}.cpp", OUT / f"{name}.o", ["-fsingle-precision-constant"]))
    jobs.append((HERE / "ref_driver.cpp", OUT / "ref_driver.o", []))

    def cc(job):
        src, obj, extra = job
        cmd = ["g++", *CXXFLAGS, *extra, f"-I{HERE}", "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError(f"{' '.join(cmd)}\n{r.stderr}")
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        objs = list(ex.map(cc, jobs))
    cmd = ["g++", "-shared", "-fopenmp", "-o", str(LIB), *map(str, objs)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError(f"{' '.join(cmd)}\n{r.stderr}")
    return LIB


def build(force: bool = False) -> Path | None:
    """Build oracle/_ref/libwcref.so. Returns None when neither the reference checkout nor
    previously generated sources are available."""
    root = reference_root()
    if root is not None:
        generate(root)  # cheap; keeps gen/ in step with the checkout
    if not all((GEN / f"{n}.cpp").is_file() for n, _ in SHADERS):
        return None
    return compile_lib()


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args()
    lib = build(a.force)
    if lib is None:
        print("reference shaders not found; nothing built", file=sys.stderr)
        sys.exit(1)
    print(lib)
