"""Recipe: compile the reference's own C sources into oracle/_ref/ (test infrastructure).

The reference (zhrv/charm_3d) needs p4est, libsc, yaml-cpp and MPI, none of
which exist in this build environment.  Its time-step arithmetic, however,
lives entirely in its own C files.  This script compiles those files
unmodified with gcc (-O2, as the reference's CMakeLists.txt:12 does) against
the p4est-subset shim in oracle/p4est_shim/, together with the driver
oracle/ref_driver.c, into two shared libraries:

  oracle/_ref/libcharm_ref.so          the reference as written
  oracle/_ref/libcharm_ref_patched.so  the same, with one change in a copy of
                                       src/limiters/charm_limiter_bj.c: the
                                       hanging-face branch also stores the
                                       species means (the original leaves those
                                       limiter slots stale, :174-193)
  oracle/_ref/libcharm_ref_plugin.so   the reference plus the GPU model plugin
                                       (charm_3d_gb300/csrc/plugin), linked to
                                       libcharm_gpu.so, to test the drop-in
                                       boundary against the reference's types

Sources are read from the reference checkout (default /root/reference, or
$CHARM_REFERENCE); nothing is copied into the repository.  Outputs go to
oracle/_ref/, which is git-ignored.  Files left out of the build: the YAML
reader (yaml-cpp), the mesh reader, VTK output and main (not on the path).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_ref")

REF_SOURCES = [
    "src/charm_globals.c",
    "src/charm_base_func.c",
    "src/charm_geom.c",
    "src/charm_eos.c",
    "src/charm_fluxes.c",
    "src/charm_bnd_cond.c",
    "src/limiters/charm_limiter.c",
    "src/limiters/charm_limiter_bj.c",
    "src/models/euler/charm_model.c",
    "src/models/ns/charm_model.c",
    "src/models/ns/charm_model_ns_conv.c",
    "src/models/ns/charm_model_ns_diff.c",
    "src/models/ns/charm_model_ns_diff_grad.c",
    "src/models/ns/charm_model_ns_diff_integrals.c",
    "src/models/ns/charm_model_ns_chem.c",
    "src/charm_amr.c",
    "src/charm_timesteps.c",
    "src/charm_init.c",
]


def reference_root() -> str | None:
    root = os.environ.get("CHARM_REFERENCE", "/root/reference")
    return root if os.path.isfile(os.path.join(root, "src", "charm_fluxes.c")) else None


def _patched_limiter(ref: str) -> str:
    """Write the one-change copy of the BJ limiter into oracle/_ref/patched/."""
    src = open(os.path.join(ref, "src/limiters/charm_limiter_bj.c")).read()
    a = "udata[f_side]->par.l.re[j] = cons[h_side].re;"
    b = "udata[h_side]->par.l.re[k] = cons[f_side].re;"
    if src.count(a) != 1 or src.count(b) != 1:
        raise RuntimeError("charm_limiter_bj.c does not have the expected hanging-face branch")
    src = src.replace(a, a + " for (cj = 0; cj < c_count; cj++) udata[f_side]->par.l.rc[cj][j] = cons[h_side].rc[cj];")
    src = src.replace(b, b + " for (cj = 0; cj < c_count; cj++) udata[h_side]->par.l.rc[cj][k] = cons[f_side].rc[cj];")
    d = os.path.join(OUT, "patched")
    os.makedirs(d, exist_ok=True)
    path = os.path.join(d, "charm_limiter_bj.c")
    with open(path, "w") as fh:
        fh.write("/* generated by oracle/build_ref.py: hanging-face species slots filled */\n" + src)
    return path


def _compile(args: tuple[list[str], str]) -> None:
    cmd, _ = args
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(" ".join(cmd) + "\n" + res.stderr)


def build(force: bool = False) -> dict[str, str]:
    ref = reference_root()
    if ref is None:
        raise FileNotFoundError("reference sources not found (set CHARM_REFERENCE)")
    libs = {"ref": os.path.join(OUT, "libcharm_ref.so"), "patched": os.path.join(OUT, "libcharm_ref_patched.so"),
            "plugin": os.path.join(OUT, "libcharm_ref_plugin.so")}
    plugin_src = os.path.join(ROOT, "charm_3d_gb300", "csrc", "plugin", "charm_model_gpu.c")
    glue_src = os.path.join(HERE, "ref_plugin_glue.c")
    ours = [os.path.join(HERE, "p4est_shim", "p4est_shim.c"), os.path.join(HERE, "ref_driver.c"),
            os.path.join(ROOT, "charm_3d_gb300", "csrc", "host", "charm_forest.c"),
            os.path.join(ROOT, "charm_3d_gb300", "csrc", "host", "charm_conn.c")]
    deps = ours + [os.path.join(HERE, "p4est_shim", f) for f in os.listdir(os.path.join(HERE, "p4est_shim"))]
    deps += [__file__, plugin_src, glue_src]
    if not force and all(os.path.exists(p) for p in libs.values()):
        if min(os.path.getmtime(p) for p in libs.values()) >= max(os.path.getmtime(p) for p in deps):
            return libs
    os.makedirs(os.path.join(OUT, "obj"), exist_ok=True)
    inc = ["-I" + os.path.join(HERE, "p4est_shim"), "-I" + os.path.join(ref, "include"),
           "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "charm_3d_gb300", "csrc", "host")]
    flags = ["gcc", "-O2", "-std=gnu99", "-fPIC", "-ffp-contract=off", "-w", "-c"]
    jobs = []
    objs_ref, objs_pat = [], []
    for rel in REF_SOURCES:
        obj = os.path.join(OUT, "obj", rel.replace("/", "_") + ".o")
        jobs.append((flags + [os.path.join(ref, rel), "-o", obj] + inc, obj))
        objs_ref.append(obj)
        if rel != "src/limiters/charm_limiter_bj.c":
            objs_pat.append(obj)
    pat_src = _patched_limiter(ref)
    pat_obj = os.path.join(OUT, "obj", "patched_charm_limiter_bj.o")
    jobs.append((flags + [pat_src, "-o", pat_obj] + inc, pat_obj))
    objs_pat.append(pat_obj)
    for src in ours:
        obj = os.path.join(OUT, "obj", os.path.basename(src) + ".o")
        jobs.append((flags + [src, "-o", obj] + inc, obj))
        objs_ref.append(obj)
        objs_pat.append(obj)
    objs_plug = []
    for src in (plugin_src, glue_src):
        obj = os.path.join(OUT, "obj", os.path.basename(src) + ".o")
        jobs.append((flags + [src, "-o", obj] + inc, obj))
        objs_plug.append(obj)
    with cf.ThreadPoolExecutor(max_workers=8) as ex:
        list(ex.map(_compile, jobs))
    for key, objs in (("ref", objs_ref), ("patched", objs_pat)):
        _compile((["gcc", "-shared", "-o", libs[key]] + objs + ["-lm"], libs[key]))
    gpu_dir = os.path.join(ROOT, "charm_3d_gb300")
    _compile((["gcc", "-shared", "-o", libs["plugin"]] + objs_ref + objs_plug +
              ["-L" + gpu_dir, "-lcharm_gpu", "-Wl,-rpath," + gpu_dir, "-lm"], libs["plugin"]))
    return libs


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
