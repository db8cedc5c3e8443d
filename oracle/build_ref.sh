#!/bin/sh
# TEST INFRASTRUCTURE: compile the reference's own C extension `_common`
# (pypybox2d/src/*.c, the float64 Vec2/Mat22/Transform/AABB types) from the
# sources where they lie, into oracle/_ref/.  Used only by
# tests/golden/make_golden.py, which runs the Python reference in this
# container to produce the golden vectors.  The build mirrors the reference's
# setup.py extension (setup.py:43-54) without its networked bootstrap; no
# FMA contraction, as the x86-64 default.
set -e
# REF: the reference source tree (required)
: "${REF:?set REF to the pypybox2d source tree}"
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
mkdir -p "$OUT"
PYINC=$(python3 -c "import sysconfig; print(sysconfig.get_paths()['include'])")
EXT=$(python3 -c "import sysconfig; print(sysconfig.get_config_var('EXT_SUFFIX'))")
gcc -O2 -fPIC -shared -ffp-contract=off -I"$PYINC" "$REF"/pypybox2d/src/*.c -o "$OUT/_common$EXT" -lm
echo "$OUT/_common$EXT"
