"""The C ABI library loads and exports every entry point include/*.h declares, and the Lighthouse 2 plugin
header compiles with the struct layouts of lib/RenderSystem/common_classes.h. No GPU work is done."""
import ctypes as C
import os
import re
import subprocess

import numpy as np

from lighthouse2_gb300 import scenes as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in ("lh2g.h", "lh2_core_api.h"):
        src = open(os.path.join(ROOT, "include", h)).read()
        names |= set(re.findall(r"LH2G_API\s+[\w:\*\s]+?\b(\w+)\s*\(", src))
    return names


def test_exports(core_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", core_lib], capture_output=True, text=True, check=True).stdout
    exported = {l.split()[-1] for l in out.splitlines() if " T " in l}
    missing = declared_symbols() - exported
    assert not missing, missing
    assert {"CreateCore", "lh2g_render_noalloc", "lh2g_trace", "lh2g_render_ex"} <= exported
    C.CDLL(core_lib)  # loads


def _signatures():
    """(return type, argument declarations) of every lh2g_* entry point of include/lh2g.h"""
    src = re.sub(r"/\*.*?\*/", "", open(os.path.join(ROOT, "include", "lh2g.h")).read(), flags=re.S)
    sigs = {}
    for m in re.finditer(r"LH2G_API\s+([\w\s\*]+?)\s*\b(lh2g_\w+)\s*\(([^)]*)\)\s*;", src):
        sigs[m.group(2)] = (m.group(1).strip(), [a.strip() for a in m.group(3).split(",") if a.strip() not in ("", "void")])
    return sigs


def test_null_handles_refused(core_lib):
    """Every entry point that takes a context, server or cache handle returns an error status for a NULL handle
    with all other arguments NULL or zero, before any CUDA call (so it runs without a GPU); the two host-only
    helpers return 0 records for empty input. The constructors and the GPU self-test are left out."""
    lib = C.CDLL(core_lib)   # a handle of its own: no argument types set elsewhere
    sigs = _signatures()
    assert len(sigs) >= 60
    skip = {"lh2g_create", "lh2g_server_create", "lh2g_nrc_create", "lh2g_nrc_wait_selftest"}
    for name, (ret, args) in sigs.items():
        if name in skip:
            continue
        f = getattr(lib, name)
        vals = []
        for a in args:
            if "*" in a:
                vals.append(C.c_void_p(None))
            elif a.startswith("double"):
                vals.append(C.c_double(0.0))
            elif a.startswith("float"):
                vals.append(C.c_float(0.0))
            elif "long long" in a:
                vals.append(C.c_longlong(0))
            else:
                vals.append(C.c_int(0))
        f.restype = C.c_void_p if ret.endswith("*") else C.c_int
        r = f(*vals)
        if name.endswith("last_error") or ret.endswith("*"):
            continue   # a message or a device pointer; it must only not crash
        if name in ("lh2g_pack_materials", "lh2g_build_light_tree"):
            assert r == 0, name
        else:
            assert r != 0, f"{name} accepted a NULL handle"


def test_pack_materials_matches_oracle(core_lib, oracle_lib):
    from lighthouse2_gb300.core import load_library
    lib = load_library()
    sc = S.spheres_2m(n_spheres=2, slices=8, stacks=6, tex_size=32)
    mats = np.ascontiguousarray(sc.materials)
    td, keep = __import__("lighthouse2_gb300.core", fromlist=["texture_descs"]).texture_descs(sc.textures)
    out = np.zeros((len(mats), 32), np.uint32)
    assert lib.lh2g_pack_materials(mats.ctypes.data, len(mats), td.ctypes.data, len(sc.textures), out.ctypes.data) == 0
    o = oracle_lib.Oracle()
    assert np.array_equal(out, oracle_lib.pack_materials(o, sc))


def test_plugin_header_and_loader(core_lib, tmp_path):
    """Loads the core exactly like lib/RenderSystem/core_api_base.cpp:97-127 (dlopen + dlsym CreateCore)."""
    src = tmp_path / "probe.cpp"
    src.write_text(r'''
#include <dlfcn.h>
#include <cstdio>
#include "lh2_core_api.h"
using namespace lighthouse2;
static_assert(sizeof(CoreTri) == 208, "CoreTri");
static_assert(sizeof(CoreLightTri) == 96 && sizeof(CorePointLight) == 32 && sizeof(CoreSpotLight) == 48, "lights");
static_assert(sizeof(CoreDirectionalLight) == 32 && sizeof(ViewPyramid) == 68 && sizeof(mat4) == 64, "view");
static_assert(sizeof(CoreTexDesc) == 40 && sizeof(CoreMaterial::Vec3Value) == 48 && sizeof(CoreMaterial::ScalarValue) == 40, "material");
static_assert(sizeof(lh2g_material) == 196 && sizeof(lh2g_gpu_material) == 128 && sizeof(lh2g_render_params) == 56 && sizeof(lh2g_filter_params) == 104, "abi");
int main(int argc, char** argv) {
    void* m = dlopen(argv[1], RTLD_NOW | RTLD_GLOBAL);
    if (!m) { printf("dlopen failed: %s\n", dlerror()); return 1; }
    typedef CoreAPI_Base* (*createCoreFunction)();
    createCoreFunction f = (createCoreFunction)dlsym(m, "CreateCore");
    if (!f) return 2;
    CoreAPI_Base* core = f();   /* Init() would create the CUDA context: not called without a GPU */
    printf("ok %d\n", core != nullptr);
    return core ? 0 : 3;
}
''')
    exe = tmp_path / "probe"
    cuda_inc = "/usr/local/cuda/include"
    subprocess.run(["g++", "-std=c++17", "-I", os.path.join(ROOT, "include"), "-I", cuda_inc, str(src), "-o", str(exe), "-ldl"], check=True)
    r = subprocess.run([str(exe), core_lib], capture_output=True, text=True)
    assert r.returncode == 0 and "ok 1" in r.stdout, r.stdout + r.stderr
