#!/bin/sh
# Compiles the reference's header-only CPU BK1, BK3 and BK5 kernels and Lagrange basis (read
# in place from the reference checkout) with oracle/ref_driver.cc into
# oracle/_ref/libref_bk5.so.  Test infrastructure only; needs the reference
# sources, so it runs where they exist and is skipped elsewhere.
set -e
here=$(cd "$(dirname "$0")" && pwd)
ref=${MFGB_REFERENCE_ROOT:-/root/reference}
if [ ! -d "$ref/CEED_BK/include" ]; then
  echo "reference sources not found at $ref; skipping oracle/_ref" >&2
  exit 0
fi
mkdir -p "$here/_ref"
g++ -O2 -fPIC -shared -std=c++17 -I"$ref/CEED_BK/include" -I"$ref/sum_factorization/include" \
    "$here/ref_driver.cc" -o "$here/_ref/libref_bk5.so"
