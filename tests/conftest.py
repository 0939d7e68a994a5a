import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built libgeye_dpm.so")


@pytest.fixture(scope="session")
def model_dir(tmp_path_factory):
    return str(tmp_path_factory.mktemp("models"))


@pytest.fixture(scope="session")
def car_paths(model_dir):
    from geye_gb300 import synth
    return synth.write_model_csv(synth.CAR_SPEC, model_dir)


@pytest.fixture(scope="session")
def person_paths(model_dir):
    from geye_gb300 import synth
    return synth.write_model_csv(synth.PERSON_SPEC, model_dir)
