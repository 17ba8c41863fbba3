"""The C-ABI library builds, loads and exports every symbol the header declares; host logic of the mirror (CPU only)."""
import re
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "ndtensors_gb300.h"


def _declared():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:nd_status|const char \*)\s*(nd_[a-z0-9_]+)\s*\(", text, re.M)))


@pytest.fixture(scope="module")
def libpath():
    sys.path.insert(0, str(ROOT / "itensors.jl_gb300"))
    import build
    return build.build()


def test_header_declares_entry_points():
    names = _declared()
    for must in ("nd_create", "nd_permutedims_f64", "nd_contract_dense_f64", "nd_bs_plan_create",
                 "nd_bs_contract_f64", "nd_bs_contract_adjoint_f64", "nd_bs_svd_f64", "nd_bs_qr_f64"):
        assert must in names


def test_library_exports_every_declared_symbol(libpath):
    out = subprocess.run(["nm", "-D", "--defined-only", str(libpath)], capture_output=True, text=True, check=True)
    exported = set(re.findall(r"\bT (nd_[a-z0-9_]+)$", out.stdout, re.M))
    missing = [n for n in _declared() if n not in exported]
    assert not missing, missing


def test_ctypes_binding_matches_header(libpath):
    import ndtensors_gb300._lib as L
    assert sorted(L.SIGNATURES) == _declared()
    lib = L.load()                      # loads without a GPU; no compute call is made
    for n in _declared():
        assert hasattr(lib, n)


def test_no_gpu_means_loud_failure():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import ndtensors_gb300 as nd
    with pytest.raises(RuntimeError):
        nd.handle(0)


def test_host_mirror_labels_and_offsets():
    import ndtensors_gb300 as nd
    assert nd.contract_labels((1, -1, 2), (-1, 3)) == (1, 2, 3)
    offs, nnz = nd.blockoffsets([(1, 2), (2, 1)], [(2, 3), (4, 5)])
    assert offs == [0, 10] and nnz == 22


def test_spectrum_kats():
    """Spectrum identities of test/base/test_decomp.jl:448-455 (host logic)."""
    import math
    import ndtensors_gb300 as nd
    assert nd.entropy(nd.Spectrum([0.5, 0.5], 0.0)) == math.log(2)
    assert nd.entropy(nd.Spectrum([1.0], 0.0)) == 0.0
    assert nd.entropy(nd.Spectrum([0.0], 0.0)) == 0.0
    assert nd.eigs(nd.Spectrum(None, 1.0)) is None
    with pytest.raises(RuntimeError):
        nd.entropy(nd.Spectrum(None, 1.0))
    assert nd.truncerror(nd.Spectrum(None, 1.0)) == 1.0
