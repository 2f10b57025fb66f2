#!/bin/sh
# Builds oracle/_ref/libmtref.so: the reference's own hot-path routines (osmanovicdino/mtcode),
# compiled straight from the reference sources through the extern "C" shim ref_driver.cpp.
# Serial (no -fopenmp): the reference's OpenMP force scatter races.  Usage:
#   oracle/build_ref.sh <reference root>     (the directory that holds Code/)
set -e
REF="${1:?usage: build_ref.sh <reference root>}"
HERE="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$HERE/_ref"
g++ -std=c++17 -O2 -w -fPIC -shared -ffp-contract=off -I"$REF/Code" \
    "$HERE/ref_driver.cpp" -o "$HERE/_ref/libmtref.so"
