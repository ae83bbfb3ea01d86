#!/bin/sh
# Builds the CPU oracle (test infrastructure) into oracle/liboracle_ppr.so.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
${CC:-gcc} -O2 -ffp-contract=off -fPIC -shared -pthread -std=gnu99 \
  "$HERE/oracle_ppr.c" "$HERE/oracle_synth.c" -o "$HERE/liboracle_ppr.so" -lm
echo "built $HERE/liboracle_ppr.so"
