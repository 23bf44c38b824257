"""Build oracle/_ref/libref.so: the reference's own step shaders, translated
mechanically to C++ (oracle/wgsl2cpp.py) from the WGSL files in the reference
tree, driven by ref_driver.cpp with the dispatch sequence of
SphSimulation3DGrid::step() (src/simulation/sph_3d_grid.rs:1261-1444).

TEST INFRASTRUCTURE ONLY. The reference tree ($FLUID_TOY_REFERENCE, or the
checkout named `reference` beside this repository) is read where it lies;
outputs go only to oracle/_ref/ (git-ignored). When the reference sources are absent (the
GPU machine) but a translation made earlier is present in oracle/_ref/, only
the C++ compile step runs.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"


def reference_root() -> Path:
    """The fluid-toy checkout the translation reads: $FLUID_TOY_REFERENCE if
    set, else a checkout named `reference` beside this repository."""
    env = os.environ.get("FLUID_TOY_REFERENCE")
    return Path(env) if env else HERE.parent.parent / "reference"


REF_SHADERS = reference_root() / "src" / "shaders"

# (namespace, shader file, prepend container_common.wgsl) — the prepend list
# follows sph_3d_grid.rs:169-193
SHADERS = [
    ("grid_clear", "grid_clear.wgsl", False),
    ("grid_build", "grid_build.wgsl", False),
    ("prefix_scan", "prefix_scan.wgsl", False),
    ("grid_reorder", "grid_reorder.wgsl", False),
    ("sph_density", "sph_density_3d_grid.wgsl", True),
    ("xsph", "xsph.wgsl", False),
    ("sph_force", "sph_force_3d_grid.wgsl", False),
    ("pcisph_predict", "pcisph_predict.wgsl", False),
    ("pcisph_solve", "pcisph_solve.wgsl", False),
    ("pcisph_finalize", "pcisph_finalize.wgsl", False),
    ("sph_integrate", "sph_integrate_3d.wgsl", True),
    # the MC density splat (marching_cubes.rs:663-669 prepends container_common)
    ("mc_density", "mc_density.wgsl", True),
    # whitewater (spray.rs:52 compiles spray_emit alone; spray_simulate expects
    # container_common prepended)
    ("spray_emit", "spray_emit.wgsl", False),
    ("spray_simulate", "spray_simulate.wgsl", True),
]

CXXFLAGS = ["-std=c++20", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fno-strict-aliasing",
            "-fPIC", "-shared", "-pthread", "-w"]


def translate_all() -> bool:
    if not REF_SHADERS.exists():
        return False
    sys.path.insert(0, str(HERE))
    from wgsl2cpp import translate
    common = (REF_SHADERS / "container_common.wgsl").read_text()
    parts = ["// generated by oracle/wgsl2cpp.py from the reference's WGSL; do not edit",
             "#pragma once", '#include "../ref_runtime.hpp"']
    for ns, fname, prepend in SHADERS:
        src = (REF_SHADERS / fname).read_text()
        if prepend:
            src = common + "\n" + src
        parts.append(f"// ---- {fname}")
        parts.append(translate(src, ns))
    OUT.mkdir(exist_ok=True)
    text = "\n\n".join(parts) + "\n"
    dst = OUT / "ref_shaders.hpp"
    if not dst.exists() or dst.read_text() != text:
        dst.write_text(text)
    return True


# The reference's host-side functions on the step's path, translated from its
# Rust sources by oracle/rs2cpp.py: (file, structs, enums, functions).
HOST_FILES = ["src/state/simulation.rs", "src/state/rigid_body.rs", "src/simulation/particle.rs",
              "src/simulation/sph_3d_grid.rs"]
HOST_ENUMS = ["ContainerStyle", "RigidBodyShape"]
HOST_STRUCTS = ["ContainerConfig", "SphConfig", "GpuSphParams3D", "GpuContainerGeometry",
                "RigidBodyConfig", "GpuRigidBody", "GpuRigidBodyAccum", "SphParticle3D",
                "GpuGridParams"]
HOST_FNS = [
    "compute_rest_density", "compute_pcisph_delta",             # simulation.rs:402-480
    "SphConfig::rest_density", "SphConfig::to_gpu_params_3d",   # :308-337
    "ContainerConfig::rotation_matrices", "ContainerConfig::to_gpu_geometry",  # :137-184
    "ContainerConfig::half_width", "ContainerConfig::half_depth",
    "RigidBodyShape::volume", "RigidBodyShape::moment_of_inertia",  # rigid_body.rs:28-80
    "RigidBodyConfig::to_gpu_rigid_body",                       # :131-146
    "quat_normalize", "quat_mul", "quat_to_rotation_rows",      # :166-205
    "integrate_rigid_body", "rotated_aabb_half_extents",        # :277-396
    "clamp_rigid_body_to_container",                            # :400-479
    "SphParticle3D::new",                                       # particle.rs:19-31
    "SphSimulation3DGrid::spawn_particles",                     # sph_3d_grid.rs:1534-1569
]


def translate_host() -> bool:
    root = reference_root()
    if not all((root / f).exists() for f in HOST_FILES):
        return False
    sys.path.insert(0, str(HERE))
    from rs2cpp import Translator, parse_file
    mods = [parse_file(root / f) for f in HOST_FILES]
    body = Translator(mods).translate(HOST_STRUCTS, HOST_ENUMS, HOST_FNS, "refhost",
                                      after_structs='#include "../ref_host_shims.hpp"')
    text = ("// generated by oracle/rs2cpp.py from the reference's Rust sources; do not edit\n"
            "#pragma once\n#include \"../rs_runtime.hpp\"\n\n" + body)
    OUT.mkdir(exist_ok=True)
    dst = OUT / "ref_host.hpp"
    if not dst.exists() or dst.read_text() != text:
        dst.write_text(text)
    return True


def build_host(quiet: bool = False, force: bool = False) -> Path | None:
    """oracle/_ref/libref_host.so: the translated host functions behind the C
    ABI of ref_host_driver.cpp."""
    translated = translate_host()
    hdr = OUT / "ref_host.hpp"
    if not hdr.exists():
        return None
    lib = OUT / "libref_host.so"
    deps = [hdr, HERE / "ref_host_driver.cpp", HERE / "rs_runtime.hpp",
            HERE / "ref_host_shims.hpp"]
    if lib.exists() and not force and all(lib.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return lib
    cxx = shutil.which("g++") or "c++"
    tmp = lib.with_suffix(".so.tmp")
    r = subprocess.run([cxx, "-std=c++20", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC",
                        "-shared", "-I", str(OUT), "-o", str(tmp),
                        str(HERE / "ref_host_driver.cpp")], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"host translation failed to compile:\n{r.stderr[-4000:]}")
    os.replace(tmp, lib)
    if not quiet:
        print(f"built {lib} ({'translated now' if translated else 'from an earlier translation'})")
    return lib


def build(quiet: bool = False, force: bool = False) -> Path | None:
    build_host(quiet, force)
    translated = translate_all()
    hdr = OUT / "ref_shaders.hpp"
    if not hdr.exists():
        if not quiet:
            print("reference shaders not available; oracle/_ref not built", file=sys.stderr)
        return None
    lib = OUT / "libref.so"
    deps = [hdr, HERE / "ref_driver.cpp", HERE / "ref_runtime.hpp"]
    if lib.exists() and not force and all(lib.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return lib
    cxx = shutil.which("g++") or "c++"
    tmp = lib.with_suffix(".so.tmp")
    r = subprocess.run([cxx, *CXXFLAGS, "-I", str(OUT), "-o", str(tmp), str(HERE / "ref_driver.cpp")],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference translation failed to compile:\n{r.stderr[-4000:]}")
    os.replace(tmp, lib)
    if not quiet:
        print(f"built {lib} ({'translated now' if translated else 'from an earlier translation'})")
    return lib


if __name__ == "__main__":
    build(force="--force" in sys.argv)
