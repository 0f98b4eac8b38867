"""The C-ABI library loads and exports every entry point include/*.h declares (CPU only)."""
import re
import shutil
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols(header="wfs.h"):
    text = (ROOT / "include" / header).read_text()
    return sorted(set(re.findall(r"^(?:int|int64_t|const char\*)\s+(wfs_\w+)\s*\(", text, flags=re.M)))


def all_declared_symbols():
    return sorted(s for h in sorted(p.name for p in (ROOT / "include").glob("*.h")) for s in declared_symbols(h))


def test_header_matches_binding_list():
    from wavefunctionsimpython_gb300 import _lib

    assert declared_symbols("wfs.h") == sorted(_lib.EXPORTED)
    assert declared_symbols("wfs_fno.h") == sorted(_lib.FNO_EXPORTED)


def test_library_exports_every_declared_symbol():
    if shutil.which("nvcc") is None and not Path("/usr/local/cuda/bin/nvcc").exists():
        pytest.skip("nvcc is not available to build the engine")
    from wavefunctionsimpython_gb300 import _lib, build_ext

    build_ext.build()
    lib = _lib.load()
    for name in all_declared_symbols():
        assert hasattr(lib, name), name
    assert lib.wfs_abi_version() == 1


def test_create_without_gpu_reports_error():
    """On a machine without a GPU, wfs_create returns an error code instead of crashing."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from wavefunctionsimpython_gb300 import Engine, WfsError, build_ext

    build_ext.build()
    with pytest.raises(WfsError):
        Engine((16, 16, 16), (1.0, 1.0, 1.0))


def test_host_only_limits_validate_arguments():
    """The wait-limit setters touch no device: out-of-range values are refused on any machine."""
    if shutil.which("nvcc") is None and not Path("/usr/local/cuda/bin/nvcc").exists():
        pytest.skip("nvcc is not available to build the engine")
    from wavefunctionsimpython_gb300 import _lib, build_ext

    build_ext.build()
    lib = _lib.load()
    assert lib.wfs_fno_set_wait_limit(-1.0) != 0
    assert lib.wfs_fno_set_wait_limit(61.0) != 0
    assert lib.wfs_fno_set_wait_limit(float("nan")) != 0
    assert lib.wfs_fno_set_wait_limit(1.0) == 0
