#!/usr/bin/env bash
# ORACLE (test infrastructure only).  Builds the reference-side checker into
# oracle/_ref/ from the reference sources where they lie (SVM_REFERENCE_DIR,
# default: a directory named "reference" beside the repository); nothing from
# the reference tree is copied into the repo.
#
#   oracle/_ref/ref_codegen          the reference's own CodeGen (codegen/codegen.cpp,
#                                    codegen/template.cpp) behind oracle/ref_codegen_shim.cpp
#   oracle/_ref/libsvm_oracle_ref.so oracle/driver.cpp compiled against the
#                                    reference's com/cpp/define.hpp + cpu-runtime.hpp
#
# The reference's generated per-query host code is then compiled by
# oracle/__init__.py with the reference's own flags (codegen/compiler.cpp:30,
# clang replaced by g++) against the same headers, into oracle/_ref/q/.
# The reference runtime header includes <xmmintrin.h>, so this builds on x86 only.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${SVM_REFERENCE_DIR:-$HERE/../../reference}"
OUT="$HERE/_ref"
if [ ! -f "$REF/codegen/codegen.cpp" ]; then
  echo "build_ref.sh: reference tree not found at $REF" >&2
  exit 3
fi
mkdir -p "$OUT/q"
printf '#include "define.hpp"\n#include "cpu-runtime.hpp"\n' > "$OUT/svm_ref_runtime.h"
g++ -w -O2 -std=c++11 -I"$REF/com/cpp" -I"$REF/codegen" \
    "$HERE/ref_codegen_shim.cpp" -o "$OUT/ref_codegen"
g++ -w -O2 -std=c++11 -fPIC -shared -pthread -I"$OUT" -I"$REF/com/cpp" \
    -DSVM_ORACLE_RUNTIME='"svm_ref_runtime.h"' "$HERE/driver.cpp" -o "$OUT/libsvm_oracle_ref.so"
echo "built $OUT"
