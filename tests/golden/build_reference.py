"""Build the reference Kwant package from its sources for fixture generation.

Test infrastructure only.  The reference's source tree is named by the
environment variable ``KWANT_REFERENCE_SRC`` (a read-only checkout of
kwant-project/kwant); this script copies its ``kwant/`` package into
``tests/golden/_refbuild/`` (git-ignored, never shipped) and compiles the
Cython extension modules the KPM path imports, with our own minimal
setuptools invocation (not the reference's ``setup.py``).  The numpy-backed
``tinyarray`` stand-in in ``tests/golden/tinyarray_standin`` replaces the
absent ``tinyarray`` dependency.

Usage::

    KWANT_REFERENCE_SRC=<kwant checkout> python tests/golden/build_reference.py
    python -c "import sys; sys.path[:0] = [...]; import kwant"

``reference_paths()`` returns the two ``sys.path`` entries that make
``import kwant`` pick up the built reference.
"""

import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REFERENCE = os.environ.get('KWANT_REFERENCE_SRC')
BUILD_DIR = os.path.join(HERE, '_refbuild')
STANDIN = os.path.join(HERE, 'tinyarray_standin')

# Cython modules that ``import kwant`` pulls in (MUMPS and SCOTCH are
# optional in the reference and absent here).
_EXTENSIONS = [
    ('kwant._system', ['kwant/_system.pyx'], ['kwant/graph']),
    ('kwant.operator', ['kwant/operator.pyx'], ['kwant/graph']),
    ('kwant.graph.core', ['kwant/graph/core.pyx'], []),
    ('kwant.graph.dijkstra', ['kwant/graph/dijkstra.pyx'], []),
    ('kwant.linalg.lapack', ['kwant/linalg/lapack.pyx'], []),
]


def reference_paths():
    return [BUILD_DIR, STANDIN]


def _built():
    return os.path.exists(os.path.join(BUILD_DIR, 'kwant', '.built'))


def build(force=False):
    if _built() and not force:
        return BUILD_DIR
    if not REFERENCE:
        raise RuntimeError('set KWANT_REFERENCE_SRC to a kwant source '
                           'checkout to build the reference')
    if not os.path.isdir(os.path.join(REFERENCE, 'kwant')):
        raise RuntimeError('reference sources not found at %s' % REFERENCE)
    import numpy as np
    from Cython.Build import cythonize
    from setuptools import Extension
    from setuptools.dist import Distribution

    if os.path.exists(BUILD_DIR):
        shutil.rmtree(BUILD_DIR)
    os.makedirs(BUILD_DIR)
    shutil.copytree(os.path.join(REFERENCE, 'kwant'),
                    os.path.join(BUILD_DIR, 'kwant'),
                    ignore=shutil.ignore_patterns('*.so', '*.c',
                                                  '__pycache__'))
    # The copied tree came from a read-only mount; make it writable.
    for root, dirs, files in os.walk(BUILD_DIR):
        for name in dirs + files:
            os.chmod(os.path.join(root, name), 0o755)

    cwd = os.getcwd()
    os.chdir(BUILD_DIR)
    try:
        exts = [Extension(name, sources,
                          include_dirs=[np.get_include()] + incs,
                          define_macros=[('NPY_NO_DEPRECATED_API',
                                          'NPY_1_7_API_VERSION')])
                for name, sources, incs in _EXTENSIONS]
        dist = Distribution({'ext_modules': cythonize(
            exts, language_level=3, quiet=True, nthreads=4)})
        cmd = dist.get_command_obj('build_ext')
        cmd.inplace = True
        cmd.parallel = 4
        dist.run_command('build_ext')
    finally:
        os.chdir(cwd)
    open(os.path.join(BUILD_DIR, 'kwant', '.built'), 'w').close()
    return BUILD_DIR


def import_reference():
    """Build if needed and import the reference ``kwant`` package."""
    build()
    for p in reversed(reference_paths()):
        if p not in sys.path:
            sys.path.insert(0, p)
    import kwant
    assert os.path.abspath(kwant.__file__).startswith(BUILD_DIR), kwant.__file__
    return kwant


if __name__ == '__main__':
    build(force='--force' in sys.argv)
    kw = import_reference()
    print('reference kwant imported from', kw.__file__)
