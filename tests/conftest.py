import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HERE = os.path.dirname(os.path.abspath(__file__))
for p in (ROOT, HERE):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_sessionstart(session):
    # the extension library is built in-tree: build it when it is missing
    # (test modules import the package, which loads it, at collection)
    lib = os.path.join(ROOT, 'kwant_gb300', 'libkwant_gb300.so')
    if not os.path.exists(lib) and not os.environ.get('KWANT_GB300_LIB'):
        from kwant_gb300 import build
        build.build()


def pytest_configure(config):
    config.addinivalue_line(
        'markers', 'gpu: needs a CUDA GPU (GB300, sm_103a) and the built '
        'extension library')


# the scratch build of the reference (fixture generation) is not part of the
# suite
collect_ignore_glob = ['golden/*']
