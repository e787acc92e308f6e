import os
import sys


ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: takes more than a few seconds on the CPU")


# Bottom-up order: the element, assembly and LU parity first, then time
# stepping, batching, serving and state files, then the cross-checks against
# fixtures, closed-form solutions and motion independence; the allocation-free
# entry point last (it shares one static scratch array).  Modules not listed
# keep their place before the listed ones.
_ORDER = ["test_oracle_kat", "test_mesh_parity", "test_abi", "test_gpu_parity", "test_lu_paths", "test_pull_force",
          "test_batch", "test_serving", "test_state_io", "test_golden", "test_closed_form", "test_motions",
          "test_patch_lu_model", "test_replicas", "test_zz_no_alloc"]


def pytest_collection_modifyitems(session, config, items):
    rank = {name: i for i, name in enumerate(_ORDER)}
    items.sort(key=lambda it: rank.get(it.module.__name__.rsplit(".", 1)[-1], -1))
