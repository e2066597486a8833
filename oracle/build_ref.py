"""Compat-build of the reference CPU ADI engine (test infrastructure only).

This script is part of the checker, not of the product. It reads the
reference's Cython/Python sources where they lie (``--reference DIR``, else the
``FDADI_REFERENCE`` environment variable, else ``/root/reference``), makes
build-time copies under ``oracle/_ref/FiniteDifference/`` (git-ignored), applies
the minimal Python-3 compatibility edits listed below, cythonizes them with
``language_level=2`` and compiles them in place. Nothing it produces is
committed; its outputs are used to pin the C restatement in
``oracle/fdadi_oracle.c`` and to generate the golden fixtures under
``tests/golden/``.

Compat edits (all made on the copies, never on the reference tree):

* ``BandedOperator.pyx``: ``import utils`` -> ``import FiniteDifference.utils
  as utils`` (implicit relative import); ``block_len = B.shape[0] /
  float(B.blocks)`` -> integer division (float slice indices were accepted by
  old numpy only, BandedOperator.pyx:685).
* ``FiniteDifferenceEngine.pyx``: ``.iteritems()`` -> ``.items()`` and
  ``sorted(...)`` of mixed int/tuple keys -> ``py2sorted`` (Python 2 ordered
  ints before tuples), ``range`` -> a list-returning, int-coercing ``range``
  (``otherdims.remove`` at :470-471 and a float count at :489).
* ``utils.py``: ``import pylab`` removed (only plotting helpers use it).
* ``Grid.py``: implicit relative imports of ``utils``/``visualize`` made
  absolute.
* ``visualize.py`` is replaced by a stub whose ``fp`` is a no-op (the original
  uses Python 2 tuple parameters, visualize.py:186).

Usage: ``python oracle/build_ref.py [--reference DIR]`` (needs Cython, run in a
container where the reference tree exists). Exits 0 and prints ``skipped`` if it
does not.

``python oracle/build_ref.py --from-generated`` compiles the C/C++ files that
an earlier run generated (already under ``oracle/_ref/``) with this machine's
compiler, Python and numpy headers, without Cython or the reference tree: the
GPU host uses this to run the reference engine as the CPU baseline.
``--auto`` does the first where the reference tree exists and the second
otherwise.
"""
import os
import re
import shutil
import subprocess
import sys

DEFAULT_REFERENCE = "/root/reference"
HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
PKG = os.path.join(OUT, "FiniteDifference")

PY2COMPAT = '''
"""Python-2 semantics needed by the reference engine under Python 3."""
import builtins as _b


def range(*args):
    return list(_b.range(*[int(a) for a in args]))


xrange = range


def _key(kv):
    k = kv[0] if isinstance(kv, tuple) and len(kv) == 2 else kv
    # Python 2 ordered numbers before tuples.
    return (0, k, ()) if not isinstance(k, tuple) else (1, 0, k)


def py2sorted(items):
    return sorted(items, key=_key)
'''

VISUALIZE_STUB = '''
def fp(*args, **kwargs):
    return None
'''


def _edit(path, subs):
    with open(path) as f:
        s = f.read()
    for pat, rep, count in subs:
        n = len(re.findall(pat, s))
        if count is not None and n != count:
            raise RuntimeError("compat edit %r matched %d times in %s (expected %d)"
                               % (pat, n, path, count))
        s = re.sub(pat, rep, s)
    with open(path, "w") as f:
        f.write(s)


def build_generated():
    """Compile the generated BandedOperator.cpp, FiniteDifferenceEngine.cpp,
    utils.c and Option.c in place (no Cython needed)."""
    import sysconfig
    srcs = {"BandedOperator": "BandedOperator.cpp",
            "FiniteDifferenceEngine": "FiniteDifferenceEngine.cpp",
            "utils": "utils.c", "Option": "Option.c"}
    if not all(os.path.exists(os.path.join(PKG, f)) for f in srcs.values()):
        print("build_ref: no generated sources, skipped")
        return 0
    suffix = sysconfig.get_config_var("EXT_SUFFIX")
    if all(os.path.exists(os.path.join(PKG, m + suffix)) for m in srcs):
        print("build_ref: already built")
        return 0
    import numpy
    inc = [sysconfig.get_paths()["include"], numpy.get_include()]
    procs = []
    for mod, src in srcs.items():
        cc = "g++" if src.endswith(".cpp") else "gcc"
        cmd = [cc, "-O2", "-w", "-shared", "-fPIC", "-ffp-contract=off"] + ["-I" + i for i in inc] + \
              [os.path.join(PKG, src), "-o", os.path.join(PKG, mod + suffix)]
        procs.append(subprocess.Popen(cmd))
    rc = max(p.wait() for p in procs)
    if rc:
        raise RuntimeError("compiling the generated reference sources failed")
    print("build_ref: built from generated sources", PKG)
    return 0


def reference_tree(argv):
    """The reference's FiniteDifference/ directory: --reference DIR, else
    $FDADI_REFERENCE, else the default location."""
    root = os.environ.get("FDADI_REFERENCE") or DEFAULT_REFERENCE
    if "--reference" in argv:
        i = argv.index("--reference")
        if i + 1 >= len(argv):
            raise SystemExit("--reference needs a directory")
        root = argv[i + 1]
    return os.path.join(root, "FiniteDifference")


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    REF = reference_tree(argv)
    if "--from-generated" in argv or ("--auto" in argv and not os.path.isdir(REF)):
        return build_generated()
    if not os.path.isdir(REF):
        print("build_ref: reference tree absent, skipped")
        return 0
    os.makedirs(PKG, exist_ok=True)
    for name in ("BandedOperator.pyx", "BandedOperator.pxd",
                 "FiniteDifferenceEngine.pyx", "utils.py", "Option.py",
                 "Grid.py", "__init__.py"):
        shutil.copy(os.path.join(REF, name), os.path.join(PKG, name))
        os.chmod(os.path.join(PKG, name), 0o644)
    with open(os.path.join(PKG, "_py2compat.py"), "w") as f:
        f.write(PY2COMPAT)
    with open(os.path.join(PKG, "visualize.py"), "w") as f:
        f.write(VISUALIZE_STUB)
    open(os.path.join(OUT, "__init__.py"), "w").close()

    header = "from FiniteDifference._py2compat import range, xrange, py2sorted\n"
    bo = os.path.join(PKG, "BandedOperator.pyx")
    _edit(bo, [
        (r"\nimport utils\n", "\nimport FiniteDifference.utils as utils\n" + header, 1),
        (r"block_len = B\.shape\[0\] / float\(B\.blocks\)",
         "block_len = B.shape[0] // B.blocks", 1),
    ])
    fde = os.path.join(PKG, "FiniteDifferenceEngine.pyx")
    _edit(fde, [
        (r"\nimport FiniteDifference\.utils as utils\n",
         "\nimport FiniteDifference.utils as utils\n" + header, 1),
        (r"sorted\(self\.operators\.iteritems\(\)\)", "py2sorted(self.operators.items())", None),
        (r"sorted\(self\.simple_operators\.items\(\)\)", "py2sorted(self.simple_operators.items())", 1),
        (r"\.iteritems\(\)", ".items()", None),
    ])
    ut = os.path.join(PKG, "utils.py")
    _edit(ut, [(r"\nimport pylab\n", "\n", 1)])
    gr = os.path.join(PKG, "Grid.py")
    _edit(gr, [
        (r"\nimport utils\n", "\nimport FiniteDifference.utils as utils\n", 1),
        (r"\nfrom utils import ", "\nfrom FiniteDifference.utils import ", 1),
        (r"\nimport visualize\n", "\nimport FiniteDifference.visualize as visualize\n", 1),
    ])

    setup_py = os.path.join(OUT, "setup_ref.py")
    with open(setup_py, "w") as f:
        f.write('''
import numpy
from setuptools import setup, Extension
from Cython.Build import cythonize
import Cython.Compiler.Options as O
O.error_on_unknown_names = False
exts = [
    Extension("FiniteDifference.BandedOperator", ["FiniteDifference/BandedOperator.pyx"],
              include_dirs=[numpy.get_include()], language="c++"),
    Extension("FiniteDifference.FiniteDifferenceEngine", ["FiniteDifference/FiniteDifferenceEngine.pyx"],
              include_dirs=[numpy.get_include()], language="c++"),
    Extension("FiniteDifference.utils", ["FiniteDifference/utils.py"]),
    Extension("FiniteDifference.Option", ["FiniteDifference/Option.py"]),
]
setup(name="fd_adi_ref", ext_modules=cythonize(exts, language_level=2, quiet=True),
      script_args=["build_ext", "--inplace", "-j", "8"])
''')
    env = dict(os.environ, CFLAGS="-O2 -w")
    subprocess.check_call([sys.executable, setup_py], cwd=OUT, env=env,
                          stdout=subprocess.DEVNULL)
    # The pure-Python copies are shadowed by the built modules; remove them so
    # the import cannot silently pick the uncompiled source.
    for name in ("utils.py", "Option.py"):
        os.remove(os.path.join(PKG, name))
    print("build_ref: built", PKG)
    return 0


if __name__ == "__main__":
    sys.exit(main())
