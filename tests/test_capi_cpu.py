"""C ABI checks that need no GPU: the library builds and loads, exports every
function include/*.h declares, and refuses to compute without a device."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

import cppirlba_gb300 as eng

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(irlba_gb300_\w+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_all_declared_symbols():
    lib = ctypes.CDLL(eng.library_path())
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_default_options_match_reference():
    o = eng._Options()
    eng.load_library().irlba_gb300_default_options(ctypes.byref(o))
    d = eng.Options()
    # Options.hpp:31-80 defaults
    assert o.invariant_subspace_tolerance == d.invariant_subspace_tolerance == -1
    assert o.convergence_tolerance == d.convergence_tolerance == 1e-5
    assert o.singular_value_ratio_tolerance == -1
    assert o.extra_work == 7 and o.max_iterations == 1000
    assert o.exact_for_small_matrix == 1 and o.exact_for_large_number == 1 and o.cap_number == 0
    assert o.seed == d.seed == 5489


def test_fails_loudly_without_gpu():
    if eng.device_count() > 0:
        pytest.skip("a GPU is visible")
    with pytest.raises(eng.IrlbaError) as e:
        eng.SimpleMatrix(np.eye(4))
    assert e.value.status == eng.ERROR_CUDA


def test_datagen_deterministic_and_dense_enough():
    from cppirlba_gb300 import datagen
    a = datagen.scrna_gene_major(50, 4000, 0.1, seed=11)
    b = datagen.scrna_gene_major(50, 4000, 0.1, seed=11)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    ptr, idx, val = a
    dens = ptr[-1] / (50 * 4000)
    assert 0.09 < dens < 0.11
    assert np.all(val >= np.log1p(1.0) - 1e-6)
    for g in range(50):
        seg = idx[ptr[g]:ptr[g + 1]]
        assert np.all(np.diff(seg) > 0) and (seg.size == 0 or (seg[0] >= 0 and seg[-1] < 4000))
    tp, ti, tv = datagen.transpose_compressed(50, 4000, ptr, idx, val)
    inp = datagen.SparseInput(4000, 50, ptr, idx, val, column_major=True)
    inp2 = datagen.SparseInput(4000, 50, tp, ti, tv, column_major=False)
    np.testing.assert_array_equal(inp.to_dense(), inp2.to_dense())


def test_operator_constructors_check_arguments_without_gpu():
    lib = eng.load_library()
    h = ctypes.c_void_p()
    for fn in (lib.irlba_gb300_matrix_create_host_operator, lib.irlba_gb300_matrix_create_device_operator):
        assert fn(10, 5, None, None, eng.FORM_FP64, ctypes.byref(h)) == eng.ERROR_INVALID_ARGUMENT
        assert "must not be NULL" in lib.irlba_gb300_last_error().decode()
    if eng.device_count() > 0:
        pytest.skip("a GPU is visible")
    with pytest.raises(eng.IrlbaError) as e:
        eng.OperatorMatrix(10, 5, lambda x: np.zeros(10), lambda y: np.zeros(5))
    assert e.value.status == eng.ERROR_CUDA
    with pytest.raises(eng.IrlbaError) as e:
        eng.DeviceOperatorMatrix(10, 5, lambda adjoint, x, y, stream: None)
    assert e.value.status == eng.ERROR_CUDA


def test_dropin_header_and_operator_example_compile(tmp_path):
    """The header-style drop-in (a user's own Matrix subclass, decorators over it,
    gpu::DeviceMatrix) and the CUDA residual-operator example build against the
    engine library without a GPU."""
    import shutil
    import subprocess
    libdir = os.path.dirname(eng.library_path())
    exe = str(tmp_path / "dropin_test")
    subprocess.run(["g++", "-std=c++17", "-O0", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "dropin_test.cpp"), "-o", exe, "-L", libdir,
                    "-lirlba_gb300", "-Wl,-rpath," + libdir], check=True)
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-c",
                    "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "residual_operator.cu"), "-o", str(tmp_path / "res.o")],
                   check=True)


def test_dropin_sparse_input_conversion(tmp_path):
    """SimpleMatrix / compute_simple / pca accept Eigen-style compressed sparse
    input (simple.hpp wraps Eigen sparse matrices too; the reference's tests
    Simple.Sparse, Compute.Sparse and Pca.Sparse use it): the conversion of
    compressed and uncompressed storage, column- and row-major, FP64 and FP32,
    into the C ABI's arrays is checked on the host."""
    import subprocess
    libdir = os.path.dirname(eng.library_path())
    exe = str(tmp_path / "sparse_input_test")
    subprocess.run(["g++", "-std=c++17", "-O0", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "sparse_input_test.cpp"), "-o", exe, "-L", libdir,
                    "-lirlba_gb300", "-Wl,-rpath," + libdir], check=True)
    out = subprocess.run([exe], check=True, stdout=subprocess.PIPE, text=True).stdout
    assert out.strip() == "ok"


def test_dropin_thread_partitions_match_oracle(tmp_path):
    """The drop-in ParallelSparseMatrix reports the reference's host thread
    partitions (get_primary_boundaries, get_secondary_boundaries,
    get_secondary_nonzero_boundaries; sparse.hpp:53-113): the header's
    computation matches the oracle's for several shapes and thread counts."""
    import json
    import subprocess
    import oracle
    libdir = os.path.dirname(eng.library_path())
    exe = str(tmp_path / "partitions_test")
    subprocess.run(["g++", "-std=c++17", "-O0", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "partitions_test.cpp"), "-o", exe, "-L", libdir,
                    "-lirlba_gb300", "-Wl,-rpath," + libdir], check=True)
    cases = json.loads(subprocess.run([exe], check=True, stdout=subprocess.PIPE, text=True).stdout)
    oracle.load()
    checked = 0
    for cs in cases:
        ptr = np.array(cs["ptr"], dtype=np.int64)
        idx = np.array(cs["idx"], dtype=np.int32)
        spec = oracle.Spec.sparse(cs["nrow"], cs["ncol"], np.ones(idx.size), idx, ptr, True, 1)
        for nt, got in cs["parts"].items():
            pb, sb, snz = oracle.partitions(spec, int(nt))
            np.testing.assert_array_equal(got["primary"], pb)
            np.testing.assert_array_equal(got["secondary"], sb)
            np.testing.assert_array_equal(np.array(got["secondary_nonzero"]).reshape(snz.shape), snz)
            checked += 1
    assert checked == 7


@pytest.mark.parametrize("custom", [False, True])
def test_dropin_parallelize_and_forwarding_header(tmp_path, custom):
    """irlba::parallelize / EigenThreadScope (parallel.hpp:32-106) through the
    reference's own header name irlba/irlba.hpp: default workers (all tasks run,
    a task's exception reaches the caller) and a caller-defined
    IRLBA_CUSTOM_PARALLEL."""
    import subprocess
    libdir = os.path.dirname(eng.library_path())
    exe = str(tmp_path / "parallel_test")
    cmd = ["g++", "-std=c++17", "-O0", "-Wall", "-Werror", "-pthread", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "parallel_test.cpp"), "-o", exe, "-L", libdir, "-lirlba_gb300",
           "-Wl,-rpath," + libdir]
    if custom:
        cmd.insert(1, "-DUSE_CUSTOM_RUNNER")
    subprocess.run(cmd, check=True)
    out = subprocess.run([exe], check=True, stdout=subprocess.PIPE, text=True).stdout
    assert out.strip() == "ok"


def test_python_sparse_input_arrays():
    """SimpleMatrix / compute_simple / pca take scipy.sparse input (the Python
    counterpart of an Eigen sparse matrix): CSC stays column-major, other
    formats become CSR, duplicates are summed and indices sorted."""
    sp = pytest.importorskip("scipy.sparse")
    rng = np.random.default_rng(4)
    dense = np.where(rng.random((30, 17)) < 0.2, rng.standard_normal((30, 17)), 0.0)
    rows, cols = np.nonzero(dense)
    # unsorted COO with a duplicate split of one entry
    order = rng.permutation(rows.size)
    r = np.concatenate([rows[order], rows[:1]])
    c = np.concatenate([cols[order], cols[:1]])
    v = np.concatenate([dense[rows[order], cols[order]], [0.5]])
    v[np.where(order == 0)[0][0]] -= 0.5
    coo = sp.coo_matrix((v, (r, c)), shape=dense.shape)
    for mat, want_cm in ((sp.csc_matrix(dense), True), (sp.csr_matrix(dense), False), (coo, False),
                         (sp.csr_matrix(dense, dtype=np.float32), False)):
        x, i, p, cm = eng.compressed_arrays(mat)
        assert cm == want_cm and i.dtype == np.int32 and p.dtype == np.int64
        assert x.dtype in (np.float32, np.float64)
        back = (sp.csc_matrix if cm else sp.csr_matrix)((x, i, p), shape=dense.shape).toarray()
        np.testing.assert_allclose(back, dense, rtol=1e-6 if x.dtype == np.float32 else 1e-15, atol=1e-15)
        for k in range(p.size - 1):
            assert np.all(np.diff(i[p[k]:p[k + 1]]) > 0)
    if eng.device_count() > 0:
        return
    with pytest.raises(eng.IrlbaError) as e:
        eng.SimpleMatrix(sp.csr_matrix(dense))
    assert e.value.status == eng.ERROR_CUDA


def test_rotation_entry_point_checks_arguments_before_the_device():
    # irlba_gb300_rotate_device validates its arguments on the host: these
    # calls return their status without touching a GPU.
    lib = eng.load_library()
    buf = (ctypes.c_double * 64)()
    p = ctypes.cast(buf, ctypes.c_void_p)
    call = lib.irlba_gb300_rotate_device
    assert call(1, p, -1, 8, 2, p, 2, 2, p, 8, None, None, 1, None) == eng.ERROR_INVALID_ARGUMENT
    assert call(1, None, 8, 8, 2, p, 2, 2, p, 8, None, None, 1, None) == eng.ERROR_INVALID_ARGUMENT
    assert call(1, p, 8, 4, 2, p, 2, 2, p, 8, None, None, 1, None) == eng.ERROR_INVALID_ARGUMENT   # ldq < L
    assert call(1, p, 8, 8, 2, p, 2, 2, p, 8, p, None, 1, None) == eng.ERROR_INVALID_ARGUMENT      # fcol, no fnorm
    assert call(1, p, 8, 8, 65, p, 65, 2, p, 8, None, None, 1, None) == eng.ERROR_UNSUPPORTED      # w > 64
    assert call(0, p, 8, 8, 2, p, 2, 65, p, 8, None, None, 1, None) == eng.ERROR_UNSUPPORTED       # k > 64
    assert "64" in lib.irlba_gb300_last_error().decode()


def test_engine_switches_are_exported_and_callable():
    eng.set_rotation_engine(0)
    eng.set_rotation_engine(1)
    eng.set_value_coding(True)
    eng.set_value_coding(False)
