#!/bin/sh
# Builds the reference's CPU paths, unmodified, from the read-only reference
# tree into oracle/_ref/ (test infrastructure only):
#   Debye      resaxslib/src/host_debye.cpp
#   PDB reader resaxslib/src/parse_pdb.cpp, utils.cpp, resaxs.cpp
#   SASA       resaxslib/src/rsasa_cpu_alg.cpp, rsasa_algorithm.cpp (dot
#              generators), with rsasa_cl_gpu_alg.cpp and
#              re_cl_algorithm_base.cpp, which the SASA factory instantiates
#              and which compile against the inert OpenCL types of shim/.
# Usage: oracle/build_ref.sh <reference_root>
#   (or RESAXS_REFERENCE_ROOT=<reference_root> oracle/build_ref.sh)
set -e
REF=${1:-$RESAXS_REFERENCE_ROOT}
[ -n "$REF" ] || { echo "usage: $0 <reference_root>" >&2; exit 2; }
HERE=$(cd "$(dirname "$0")" && pwd)
[ -f "$REF/resaxslib/src/host_debye.cpp" ] || { echo "reference not found at $REF" >&2; exit 3; }
mkdir -p "$HERE/_ref"
S="$REF/resaxslib/src"
g++ -std=c++14 -O2 -shared -fPIC -w -include limits \
    -I "$HERE/shim" -I "$REF/resaxslib/include" \
    "$HERE/ref_wrap.cpp" "$S/host_debye.cpp" \
    "$S/parse_pdb.cpp" "$S/utils.cpp" "$S/resaxs.cpp" \
    "$S/rsasa_cpu_alg.cpp" "$S/rsasa_algorithm.cpp" \
    "$S/rsasa_cl_gpu_alg.cpp" "$S/re_cl_algorithm_base.cpp" \
    -o "$HERE/_ref/libref_host_debye.so"
echo "built $HERE/_ref/libref_host_debye.so"
