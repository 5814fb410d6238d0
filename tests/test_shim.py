"""The reference-side binding compiles against IQ-TREE 2's own headers.

``iqtree2_gb300/shim/`` holds the PhyloTree translation unit that installs
the engine behind the kernel function pointers and three patches for the
reference (member declarations in tree/phylotree.h, the dispatch in
tree/phylotreesse.cpp, engine release in tree/phylotree.cpp). This test
applies the patches to copies of those files, writes an ``iqtree_config.h``
from the reference's ``iqtree_config.h.in`` and runs ``g++ -std=c++17
-fsyntax-only`` on the shim and on the patched sources. The shim's
static_asserts check that its four entry points have exactly the types of
the reference's pointers (tree/phylotree.h:899-901, 947-948, 1000-1001,
1342-1343). Needs a reference checkout (skipped without one).
"""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM = os.path.join(ROOT, "iqtree2_gb300", "shim")
REF = os.environ.get("IQTREE_REFERENCE", "/root/reference")

pytestmark = pytest.mark.skipif(not os.path.exists(os.path.join(REF, "tree", "phylotree.h")),
                                reason="no reference checkout")

PATCHED = {"phylotree_h.patch": "phylotree.h", "phylotreesse_cpp.patch": "phylotreesse.cpp",
           "phylotree_cpp.patch": "phylotree.cpp"}


def _config_header(dst):
    src = open(os.path.join(REF, "iqtree_config.h.in")).read()
    src = src.replace("@iqtree_VERSION_MAJOR@", "2").replace("@iqtree_VERSION_MINOR@", "3")
    src = src.replace('"@iqtree_VERSION_PATCH@"', '"0"')
    src = re.sub(r"#cmakedefine (HAVE_GETTIMEOFDAY|HAVE_GETRUSAGE)", r"#define \1", src)
    src = re.sub(r"#cmakedefine \w+.*", "", src)
    src = re.sub(r"@\w+@", "0", src)
    open(os.path.join(dst, "iqtree_config.h"), "w").write(src)


@pytest.fixture(scope="module")
def patched(tmp_path_factory):
    d = tmp_path_factory.mktemp("shim")
    os.makedirs(d / "tree")
    for patch, name in PATCHED.items():
        shutil.copy(os.path.join(REF, "tree", name), d / "tree" / name)
        r = subprocess.run(["patch", "-p1", "-d", str(d), "-i", os.path.join(SHIM, patch)],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
    _config_header(str(d))
    return d


def _syntax(d, src):
    cmd = ["g++", "-std=c++17", "-fsyntax-only", "-fopenmp", "-DIQTREE_GB300", "-w",
           f"-I{d}", f"-I{d}/tree", f"-I{REF}", f"-I{REF}/tree", f"-I{REF}/yaml-cpp/include",
           f"-I{os.path.join(ROOT, 'include')}", src]
    if os.uname().machine == "x86_64":
        cmd[4:4] = ["-mavx2", "-mfma"]
    return subprocess.run(cmd, capture_output=True, text=True, timeout=600)


def test_patches_apply_cleanly(patched):
    for name in PATCHED.values():
        assert "IQTREE_GB300" in open(patched / "tree" / name, newline="").read()


def test_shim_compiles_against_reference_headers(patched):
    r = _syntax(patched, os.path.join(SHIM, "phylotreegb300.cpp"))
    assert r.returncode == 0, r.stderr[-4000:]


def test_patched_dispatch_compiles(patched):
    r = _syntax(patched, str(patched / "tree" / "phylotreesse.cpp"))
    assert r.returncode == 0, r.stderr[-4000:]


def test_shim_binds_the_engine_entry_points():
    """Every engine call in the shim is one the C ABI declares."""
    src = open(os.path.join(SHIM, "phylotreegb300.cpp")).read()
    hdr = open(os.path.join(ROOT, "include", "iqgpu.h")).read()
    used = set(re.findall(r"\b(iqgpu_\w+)\s*\(", src))
    declared = set(re.findall(r"\b(iqgpu_\w+)\s*\(", hdr))
    assert used and used <= declared, used - declared
