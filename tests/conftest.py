import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "tests"))
GOLDEN = os.path.join(REPO, "tests", "golden")
CARD = os.path.join(GOLDEN, "cards", "pp_con_pipi.json")
CARD_SCR = os.path.join(GOLDEN, "cards", "pp_con_pipi_screened.json")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through the C ABI)")


@pytest.fixture(scope="session")
def params():
    from graniitti_gb300 import card
    return card.build_params(card.read_card(CARD))


@pytest.fixture(scope="session")
def params_screened():
    from graniitti_gb300 import card
    return card.build_params(card.read_card(CARD_SCR))


@pytest.fixture(scope="session")
def lib_built():
    from graniitti_gb300 import build
    return build.build_library()


@pytest.fixture(scope="session")
def gpu():
    import ctypes
    try:
        import torch
        ok = torch.cuda.is_available()
    except Exception:
        ok = False
    if not ok:
        pytest.skip("no CUDA device")
    from graniitti_gb300 import build
    build.build_library()
    return True
