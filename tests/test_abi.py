"""C-ABI checks that need no GPU: the library loads, exports every symbol
include/rhyme_gpu.h declares, its struct layout matches, and parameter
validation rejects bad input before any CUDA call."""
import ctypes as C
import os
import re

import pytest

from rhyme_gb300 import build, gpu, params

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return gpu.load()


def header_symbols():
    text = open(os.path.join(ROOT, "include", "rhyme_gpu.h")).read()
    return sorted(set(re.findall(r"\b(rhyme_gpu_\w+)\s*\(", text)))


def test_exports_every_declared_symbol(lib):
    declared = header_symbols()
    assert len(declared) >= 17
    for name in declared:
        assert hasattr(lib, name), name
    assert sorted(gpu.EXPORTS) == declared


def test_abi_version(lib):
    assert lib.rhyme_gpu_abi_version() == 1


def test_params_layout():
    # 10 ints (incl. bc[6]) + precision + sweep_tuning = 12 ints, then 7 doubles, then 30 doubles
    assert C.sizeof(gpu.Params) == 12 * 4 + 7 * 8 + 30 * 8
    # struct rhyme_gpu_request: 12 ints, omega + dx[3], cells, output and
    # shapes pointers, nshapes + reserved
    assert C.sizeof(gpu.Request) == 12 * 4 + 4 * 8 + 3 * 8 + 2 * 4
    # struct rhyme_gpu_shape: 4 ints, 6 ints, 10 + 3 + 2 + 2 + 2 + 3 + 5 doubles
    assert C.sizeof(gpu.Shape) == 10 * 4 + 27 * 8
    assert gpu.Params.gamma.offset == 48


@pytest.mark.parametrize("bad", [dict(ndim=4), dict(limiter=9), dict(solver_type=3), dict(gamma=1.0),
                                 dict(bc=[7, 2, 2, 2, 2, 2]), dict(precision=5), dict(n_iter=-1)])
def test_create_rejects_bad_params(lib, bad):
    p = params.hydro_params(2)
    p.update(bad)
    s = gpu.params_struct(p)
    h = C.c_void_p()
    rc = lib.rhyme_gpu_create(C.byref(h), C.byref(s))
    assert rc == gpu.EINVAL
    assert not h.value


def test_null_arguments(lib):
    assert lib.rhyme_gpu_create(None, None) == gpu.EINVAL
    assert lib.rhyme_gpu_synchronize(None) == gpu.EINVAL
    assert lib.rhyme_gpu_last_error(None) == b""
    assert lib.rhyme_gpu_get_rows(None, 0, 0, 1, None) == gpu.EINVAL
    assert lib.rhyme_gpu_set_rows(None, 0, 0, 1, None) == gpu.EINVAL
    assert lib.rhyme_gpu_set_host_writeback(None, 0, 1) == gpu.EINVAL


FORTRAN = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "rhyme_gb300", "fortran")


def _fortran_bindings():
    """(C names bound in rhyme_gpu_c.f90, fields of rhyme_gpu_params_t)."""
    import re
    src = open(os.path.join(FORTRAN, "rhyme_gpu_c.f90")).read()
    names = re.findall(r"bind\(c, name='(rhyme_gpu_[a-z_0-9]+)'\)", src)
    body = src[src.index("type, bind(c) :: rhyme_gpu_params_t"):src.index("end type rhyme_gpu_params_t")]
    fields = re.findall(r"(integer\(c_int\)|real\(c_double\)) :: (\w+)(?:\(([\d, ]+)\))?", body)
    return names, fields


def test_fortran_bindings_name_declared_functions():
    """The uncompiled Fortran interfaces bind only functions the header
    declares (and the library exports)."""
    names, _ = _fortran_bindings()
    assert len(names) >= 20
    assert set(names) <= set(gpu.EXPORTS), sorted(set(names) - set(gpu.EXPORTS))


def test_fortran_params_type_matches_the_c_struct():
    """rhyme_gpu_params_t has the C struct's fields in order, with the same
    kinds and element counts (Fortran inflow(5, 6) is C inflow[6][5])."""
    _, fields = _fortran_bindings()
    got = []
    for kind, name, dims in fields:
        n = 1
        for d in (dims.split(",") if dims else []):
            n *= int(d)
        got.append((name, "int" if kind.startswith("integer") else "double", n))
    want = []
    for name, ctype in gpu.Params._fields_:
        n = C.sizeof(ctype)
        base = "double" if "double" in repr(ctype) else "int"
        want.append((name, base, n // (8 if base == "double" else 4)))
    assert got == want



@pytest.mark.parametrize("compiler,flags", [("gcc", ["-std=c99", "-x", "c"]),
                                            ("g++", ["-std=c++11", "-x", "c++"])])
def test_header_is_plain_c_and_a_c_driver_links(lib, tmp_path, compiler, flags):
    """tests/c_abi_driver.c (the driver loop of src/main.f90:106-177 in C)
    compiles with warnings as errors as strict C99 and as C++, and links
    against the built library: every entry point it calls resolves."""
    import shutil
    import subprocess
    if shutil.which(compiler) is None:
        pytest.skip("%s not found" % compiler)
    src = os.path.join(ROOT, "tests", "c_abi_driver.c")
    obj = str(tmp_path / "driver.o")
    cmd = [compiler] + flags + ["-Wall", "-Wextra", "-Werror", "-pedantic",
                                "-I", os.path.join(ROOT, "include"), "-c", src, "-o", obj]
    out = subprocess.run(cmd, capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    exe = str(tmp_path / "driver")
    out = subprocess.run([compiler, obj, "-L", build.OUT_DIR, "-lrhyme_gpu", "-o", exe],
                         capture_output=True, text=True)
    assert out.returncode == 0, out.stderr


def test_product_path_fails_loudly_without_a_gpu(lib):
    """No CPU fallback: without a visible GPU, creating a context raises
    RhymeGpuError(ECUDA) (parameter validation passes, the first CUDA call
    fails); the server does the same."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    with pytest.raises(gpu.RhymeGpuError) as e:
        gpu.Context(params.hydro_params(1))
    assert e.value.code == gpu.ECUDA
    with pytest.raises(gpu.RhymeGpuError) as e:
        gpu.Server(params.hydro_params(3, precision=params.MIXED))
    assert e.value.code == gpu.ECUDA


def test_missing_library_raises_import_error(monkeypatch, tmp_path):
    """Without the built library the binding raises at load, before any
    call; nothing stands in for it."""
    monkeypatch.setattr(gpu, "_lib", None)
    monkeypatch.setattr(gpu, "LIB_PATH", str(tmp_path / "librhyme_gpu.so"))
    with pytest.raises(ImportError):
        gpu.load()
    with pytest.raises(ImportError):
        gpu.Context(params.hydro_params(1))
