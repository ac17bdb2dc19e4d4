"""Shared test set-up: import paths, the `gpu` marker, library fixtures."""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "ngp-encode-server_gb300")
for p in (os.path.join(REPO, "oracle"), PKG, REPO):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def nes_lib():
    """Builds (if needed) and loads libnes_gb300.so."""
    import nes_build
    nes_build.build()
    import nes
    nes.load()
    return nes


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.load()
    return oracle


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(scope="session")
def scene0(oracle_mod):
    return oracle_mod.Scene(0, 19)


@pytest.fixture(scope="session")
def r32(nes_lib, cuda):
    """FP32 plain-path renderer on the reference scene (seed 0, 2^19)."""
    r = nes_lib.Renderer(precision=nes_lib.PREC_FP32, max_pixels=2 * 1920 * 1832)
    yield r
    r.close()


@pytest.fixture(scope="session")
def rtc(nes_lib, cuda):
    """FP16 tensor-core renderer on the reference scene (seed 0, 2^19)."""
    r = nes_lib.Renderer(precision=nes_lib.PREC_FP16_TC, max_pixels=2 * 1920 * 1832)
    yield r
    r.close()


@pytest.fixture(params=["fp32", "tc"])
def renderer(request, nes_lib, cuda):
    """Both precisions of the reference-scene renderer."""
    return request.getfixturevalue("r32" if request.param == "fp32" else "rtc")
