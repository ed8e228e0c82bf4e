#!/usr/bin/env bash
# Builds an importable copy of the reference Brian2 (the oracle's generator) as a
# SYMLINK tree under oracle/_ref/pyenv: no reference source is copied, only
# linked, and the two Cython extensions the package needs are compiled next to
# the links.  `pyparsing` is provided by a one-line shim that re-exports the copy
# vendored inside pip.  Only a host with the reference sources can build it; the
# tree is ignored by git and left out of copies of the repository to other hosts.
#
# usage: bash oracle/make_ref_env.sh /path/to/reference
set -euo pipefail
REF=${1:?usage: make_ref_env.sh /path/to/reference (the directory holding brian2/)}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref/pyenv"
[ -d "$REF/brian2" ] || { echo "reference not found at $REF" >&2; exit 1; }
rm -rf "$OUT"
mkdir -p "$OUT"
# mirror directories, symlink files (skip shipped bytecode caches)
( cd "$REF" && find brian2 -type d -name __pycache__ -prune -o -type d -print ) | while read -r d; do mkdir -p "$OUT/$d"; done
( cd "$REF" && find brian2 -type d -name __pycache__ -prune -o -type f ! -name '*.pyc' -print ) | while read -r f; do ln -s "$REF/$f" "$OUT/$f"; done
echo "from pip._vendor.pyparsing import *  # noqa" > "$OUT/pyparsing.py"
echo "from pip._vendor.pyparsing import __version__  # noqa" >> "$OUT/pyparsing.py"
# compile the two Cython extensions (setup.py of the reference declares them)
cd "$OUT"
export PYTHONDONTWRITEBYTECODE=1
python - <<'PY'
import numpy, os
from Cython.Build import cythonize
from setuptools import Extension
from setuptools.dist import Distribution
from setuptools.command.build_ext import build_ext
exts = [Extension("brian2.synapses.cythonspikequeue", ["brian2/synapses/cythonspikequeue.pyx"],
                  include_dirs=[numpy.get_include()]),
        Extension("brian2.memory.cythondynamicarray", ["brian2/memory/cythondynamicarray.pyx"],
                  include_dirs=[numpy.get_include(), "brian2/devices/cpp_standalone/brianlib"])]
# cythonize writes .cpp next to the .pyx; the .pyx are symlinks, so write into build/ instead
exts = cythonize(exts, build_dir="_cybuild", language_level=3, quiet=True)
d = Distribution({"ext_modules": exts})
cmd = build_ext(d); cmd.inplace = 1; cmd.build_temp = "_cybuild/tmp"
cmd.ensure_finalized(); cmd.run()
PY
echo "oracle env ready: PYTHONPATH=$OUT"
