import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HERE = os.path.dirname(os.path.abspath(__file__))
for p in (ROOT, HERE):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line(
        'markers', 'gpu: needs a CUDA GPU (GB300, sm_103a) and the built '
        'extension library')


# the scratch build of the reference (fixture generation) is not part of the
# suite
collect_ignore_glob = ['golden/*']
