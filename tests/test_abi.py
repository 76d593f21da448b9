"""The C ABI surface, checked without a GPU: the in-tree library loads and
exports every function include/cajitafluids_gb300.h declares, the ctypes
binding covers exactly that list, and the ABI version matches.  No compute
call is made."""
import os
import re
import subprocess

from cajitafluids_gb300 import _lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "cajitafluids_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(cf_[a-z0-9_]+)\s*\(", text)))


def exported_symbols(path):
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True, check=True).stdout
    return sorted({ln.split()[-1] for ln in out.splitlines() if " T " in ln and ln.split()[-1].startswith("cf_")})


def test_header_declares_a_non_trivial_abi():
    fns = declared_functions()
    for must in ("cf_ctx_create", "cf_step", "cf_project", "cf_advect", "cf_add_inputs", "cf_upload",
                 "cf_download", "cf_div_norms_noalloc"):
        assert must in fns


def test_library_exports_every_declared_function(built):
    fns = declared_functions()
    syms = exported_symbols(L.LIB_PATH)
    assert fns == syms, (set(fns) ^ set(syms))


def test_binding_covers_the_abi(built):
    assert sorted(L.SIGNATURES) == declared_functions()
    lib = L.load()
    assert lib.cf_abi_version() == 1
    for name in declared_functions():
        assert hasattr(lib, name)


def test_error_codes_match_header():
    text = open(HEADER).read()
    for name in ("CF_ERR_INVALID", "CF_ERR_CUDA", "CF_ERR_UNSUPPORTED", "CF_ERR_NOT_CONVERGED", "CF_ERR_NUMERIC",
                 "CF_ERR_NOMEM", "CF_ERR_MESH", "CF_ERR_TOO_LARGE", "CF_ERR_TIMEOUT"):
        m = re.search(r"#define\s+%s\s+\((-?\d+)\)" % name, text)
        assert m, name
        assert int(m.group(1)) == getattr(L, name)


def test_missing_library_fails_loudly(tmp_path):
    """Without libcfgpu.so the binding raises; nothing falls back to a CPU
    path (run in a fresh interpreter, since the library is cached once
    loaded)."""
    import sys
    code = ("from cajitafluids_gb300 import _lib\n"
            f"_lib.load({str(tmp_path / 'libcfgpu.so')!r})\n")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, cwd=ROOT, timeout=120)
    assert r.returncode != 0
    assert "OSError" in r.stderr and "no CPU fallback" in r.stderr
