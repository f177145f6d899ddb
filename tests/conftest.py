import ctypes as ct
import os
import shutil
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU and the built library")


@pytest.fixture(scope="session")
def ctx():
    """One device context for the GPU tests (fails loudly without the CUDA library)."""
    from chrono_photo_gb300 import Context
    c = Context(0)
    yield c
    c.close()


def pytest_collection_modifyitems(config, items):
    # the pure-Python restatement divides by zero where the reference does (inf results)
    for item in items:
        item.add_marker(pytest.mark.filterwarnings("ignore::RuntimeWarning"))


@pytest.fixture(scope="session")
def mock_device_lib(tmp_path_factory):
    """The compositing server (cp_server.cpp), option preparation (cp_prepare.cpp) and memory
    accounting (cp_memory.cpp) built with g++ against the host-memory CUDA runtime of
    tests/mock_device, for CPU tests of the host logic. -Bsymbolic: the library's own runtime
    functions win over a CUDA runtime that another module (torch) has already loaded into the
    process with global symbols."""
    from chrono_photo_gb300 import _abi
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    csrc = os.path.join(ROOT, "chrono_photo_gb300", "csrc")
    mock = os.path.join(ROOT, "tests", "mock_device")
    sources = [os.path.join(csrc, f) for f in ("cp_server.cpp", "cp_prepare.cpp", "cp_memory.cpp")]
    sources.append(os.path.join(mock, "mock_device.cpp"))
    out = str(tmp_path_factory.mktemp("mock_device") / "libserver_mock.so")
    subprocess.run([gxx, "-std=c++17", "-O1", "-g", "-fPIC", "-shared", "-pthread", "-Wall",
                    "-Wl,-Bsymbolic", "-I", mock, "-o", out] + sources, check=True)
    lib = ct.CDLL(out)
    P, U64, I32 = ct.c_void_p, ct.c_uint64, ct.c_int32
    for name, res, args in (
            ("mock_ctx_create", P, [U64]), ("mock_ctx_destroy", None, [P]),
            ("mock_ctx_used", U64, [P]), ("mock_ctx_launches", U64, [P]),
            ("mock_reset", None, []), ("mock_shutdown", None, []),
            ("mock_hold", None, [ct.c_uint]), ("mock_fail_launch_words", None, [ct.c_int]),
            ("mock_fault_launches", None, [ct.c_int]),
            ("mock_fail_allocs", None, [ct.c_uint, ct.c_int]),
            ("mock_set_pool_limit", None, [U64]),
            ("mock_stats", ct.c_int, [ct.POINTER(U64), ct.c_int]),
            ("mock_wait_idle", ct.c_int, [ct.c_int]),
            ("mock_prepare", ct.c_int, [ct.POINTER(_abi.Stack), ct.POINTER(_abi.Params),
                                        ct.POINTER(I32), ct.POINTER(ct.c_float)]),
            ("cp_server_create", ct.c_int, [P, U64, I32, ct.POINTER(P)]),
            ("cp_server_submit", ct.c_int, [P, ct.POINTER(_abi.Job), ct.POINTER(U64)]),
            ("cp_server_wait", ct.c_int, [P, U64, I32, ct.POINTER(_abi.JobResult)]),
            ("cp_server_cancel", ct.c_int, [P, U64]),
            ("cp_server_destroy", ct.c_int, [P]),
            ("cp_params_default", None, [ct.POINTER(_abi.Params)]),
            ("cp_ctx_fail_allocations", ct.c_int, [P, I32]),
            ("cp_ctx_last_error", ct.c_int, [P, ct.c_char_p, ct.c_size_t])):
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib
