#!/bin/sh
# Installs the reference (dmalhotra/SCTL) into the repository's baseline/_ref
# for the CPU baseline and the drop-in tests -- BASELINE INFRASTRUCTURE ONLY.
#
#   oracle/install_ref.sh <path to an SCTL checkout>      (or SCTL_REF=<path>)
#
# SCTL is header-only C++ with no Python packaging, so `pip install --target`
# has nothing to install; the install is a copy of its include/ tree (the
# headers, sse2neon.h and experimental/quad_element.{hpp,cpp}).  baseline/_ref
# is git-ignored: the reference's sources never enter the repository's history.
set -eu
SRC="${1:-${SCTL_REF:-}}"
if [ -z "$SRC" ] || [ ! -f "$SRC/include/sctl.hpp" ]; then
  echo "usage: $0 <SCTL checkout containing include/sctl.hpp>" >&2
  exit 2
fi
HERE="$(cd "$(dirname "$0")" && pwd)"
DST="$HERE/../baseline/_ref"
mkdir -p "$DST"
rm -rf "$DST/include"
cp -R "$SRC/include" "$DST/include"
chmod -R u+w "$DST/include"
if [ -f "$SRC/LICENSE" ]; then cp "$SRC/LICENSE" "$DST/LICENSE"; fi
echo "installed $(find "$DST/include" -type f | wc -l) reference files into $DST"
