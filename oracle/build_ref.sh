#!/bin/sh
# Builds oracle/_ref/ref_driver from the reference's own headers.
# Usage: oracle/build_ref.sh [reference_root]   (default $HASHDAG_REFERENCE_ROOT, else /root/reference)
# Runs only where the reference tree exists; the output stays out of git.
set -e
REF=${1:-${HASHDAG_REFERENCE_ROOT:-/root/reference}}
HERE=$(cd "$(dirname "$0")" && pwd)
[ -f "$REF/include/hashdag/NodePool.hpp" ] || { echo "reference tree not found at $REF" >&2; exit 3; }
mkdir -p "$HERE/_ref"
g++ -std=c++20 -O2 -DNDEBUG -DHASHDAG_TEST -Wno-interference-size -ffp-contract=off \
    -I"$REF/include" -I"$REF/dep/libfork/include" -I"$REF/dep/glm/include" -I"$REF/dep/parallel-hashmap" -pthread \
    "$HERE/ref_driver.cpp" -o "$HERE/_ref/ref_driver"
