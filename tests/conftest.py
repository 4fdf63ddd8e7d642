import pathlib
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
GOLDEN = ROOT / "tests" / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libpjg.so")


@pytest.fixture(scope="session")
def golden():
    return GOLDEN


@pytest.fixture(scope="session")
def amy(golden):
    from pyjess_gb300 import Molecule

    return Molecule.load(str(golden / "1AMY.pdb"))


@pytest.fixture(scope="session")
def t133(golden):
    from pyjess_gb300 import Template

    return Template.load(str(golden / "1.3.3.tpl"))


@pytest.fixture(scope="session")
def t412(golden):
    from pyjess_gb300 import Template

    return Template.load(str(golden / "4.1.2.tpl"))


@pytest.fixture(scope="session")
def ayx(golden):
    from pyjess_gb300 import Molecule

    return Molecule.load(str(golden / "5ayx.EF.pdb"))


@pytest.fixture(scope="session")
def golden_blocks(golden):
    text = (golden / "1AMY+1.3.3.txt").read_text()
    return [b for b in text.split("REMARK") if b.strip()]
