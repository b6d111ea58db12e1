#!/bin/sh
# Builds the reference's CPU Debye path (resaxslib/src/host_debye.cpp) and its
# PDB reader (resaxslib/src/parse_pdb.cpp, utils.cpp, resaxs.cpp), unmodified,
# from the read-only reference tree into oracle/_ref/.  Test infrastructure only.
# Usage: oracle/build_ref.sh [reference_root]   (default /root/reference)
set -e
REF=${1:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
[ -f "$REF/resaxslib/src/host_debye.cpp" ] || { echo "reference not found at $REF" >&2; exit 3; }
mkdir -p "$HERE/_ref"
g++ -std=c++14 -O2 -shared -fPIC -w -include limits \
    -I "$HERE/shim" -I "$REF/resaxslib/include" \
    "$HERE/ref_wrap.cpp" "$REF/resaxslib/src/host_debye.cpp" \
    "$REF/resaxslib/src/parse_pdb.cpp" "$REF/resaxslib/src/utils.cpp" \
    "$REF/resaxslib/src/resaxs.cpp" \
    -o "$HERE/_ref/libref_host_debye.so"
echo "built $HERE/_ref/libref_host_debye.so"
