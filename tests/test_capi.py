"""The C ABI library builds, loads, and exports every function the headers
in include/ declare.  No compute call is made (no GPU needed)."""
import ctypes
import glob
import os
import re

from shadowvm_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(path):
    text = re.sub(r"/\*.*?\*/", "", open(path).read(), flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    return set(re.findall(r"\b(svm_[a-z0-9_]+)\s*\(", text))


def test_library_exports_every_declared_function(built_lib):
    lib = ctypes.CDLL(built_lib)
    headers = glob.glob(os.path.join(ROOT, "include", "*.h"))
    assert headers
    names = set()
    for h in headers:
        names |= declared(h)
    assert "svm_run_pipeline" in names and "svm_init" in names
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_host_only_calls(built_lib):
    lib = capi.load(built_lib)
    assert lib.svm_abi_version() == 1
    cfg = capi.svm_config()
    lib.svm_config_default(ctypes.byref(cfg))
    assert cfg.tuple_per_bulk == 2_000_000 and cfg.join_mode == capi.JOIN_REF_COMPAT
    assert cfg.hash_char_signed == 1
    assert lib.svm_last_error(None) == b"null context"
    assert lib.svm_run_pipeline(None, None) == capi.E_INVALID_ARG


def test_headers_are_plain_c(tmp_path):
    """The boundary is a C ABI: every header compiles as strict C99 on its
    own (what a cgo, JNI or N-API stub includes), and a C program can take
    the address of every declared entry point."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        import pytest
        pytest.skip("no C compiler")
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        names = sorted(declared(h))
        src = tmp_path / "use.c"
        src.write_text(f'#include "{h}"\n' + "void *entry_points[] = {\n" +
                       "".join(f"  (void *)&{n},\n" for n in names) + "};\n")
        r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-Wno-pedantic",
                            "-fsyntax-only", str(src)], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-fsyntax-only", "-x", "c",
                            h], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


def _status_functions():
    """(name, parameter list) of every header function returning svm_status."""
    out = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for name, params in re.findall(r"\bsvm_status\s+(svm_[a-z0-9_]+)\s*\(([^)]*)\)", text):
            out.append((name, [p.strip() for p in params.split(",") if p.strip()]))
    return out


def test_every_entry_point_rejects_a_null_context(built_lib):
    """Each call that takes a context answers SVM_E_INVALID_ARG to a null one
    (and null / zero arguments) before it touches the GPU."""
    lib = ctypes.CDLL(built_lib)
    checked = 0
    for name, params in _status_functions():
        if not params or not re.match(r"(const\s+)?svm_ctx\s*\*", params[0]):
            continue
        args = []
        for p in params:
            if "*" in p:
                args.append(ctypes.c_void_p(None))
            elif "unsigned long long" in p or "uint64_t" in p or "size_t" in p:
                args.append(ctypes.c_ulonglong(0))
            else:
                args.append(ctypes.c_int(0))
        fn = getattr(lib, name)
        fn.restype = ctypes.c_int
        assert fn(*args) == capi.E_INVALID_ARG, name
        checked += 1
    assert checked >= 19


def test_init_validates_before_the_gpu(built_lib):
    lib = capi.load(built_lib)
    cfg = capi.svm_config()
    lib.svm_config_default(ctypes.byref(cfg))
    ctx = ctypes.c_void_p()
    assert lib.svm_init(ctypes.byref(cfg), None) == capi.E_INVALID_ARG
    bad = capi.svm_config()
    lib.svm_config_default(ctypes.byref(bad))
    bad.tuple_per_bulk = 0
    assert lib.svm_init(ctypes.byref(bad), ctypes.byref(ctx)) == capi.E_INVALID_ARG and not ctx.value
    lib.svm_config_default(ctypes.byref(bad))
    bad.join_mode = 7
    assert lib.svm_init(ctypes.byref(bad), ctypes.byref(ctx)) == capi.E_INVALID_ARG and not ctx.value
    # a valid configuration: a context where a GPU is present, else a CUDA error and no context
    st = lib.svm_init(ctypes.byref(cfg), ctypes.byref(ctx))
    if st == capi.OK:
        lib.svm_destroy(ctx)
    else:
        assert st == capi.E_CUDA and not ctx.value
