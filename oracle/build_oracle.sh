#!/bin/sh
# Builds the CPU oracle (test infrastructure) into oracle/libmf_oracle.so.
set -e
here=$(cd "$(dirname "$0")" && pwd)
gcc -O2 -fopenmp -fPIC -shared -std=c11 "$here/mf_oracle.c" -o "$here/libmf_oracle.so" -lm
