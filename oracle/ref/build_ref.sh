#!/usr/bin/env bash
# Builds the reference's own physics sources, unmodified, into a serial
# (no OpenMP) test-oracle executable: oracle/_ref/ref_harness.
#
# Reads the sources where they lie (REF_SRC; unset, oracle/ref/refpath.py
# locates the checkout) and
# writes nothing but oracle/_ref/. Needs only g++ and the LibTorch headers and
# libraries that ship inside the installed torch wheel.
#
#   REF_SRC=/path/to/reference/src  oracle/ref/build_ref.sh
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/../_ref"
if [ -z "${REF_SRC:-}" ]; then
  REF_SRC="$(cd "$HERE/../.." && python3 -c 'from oracle.ref.refpath import ref_src; print(ref_src() or "")')"
fi
if [ -z "$REF_SRC" ] || [ ! -d "$REF_SRC" ]; then
  echo "reference sources not found at $REF_SRC" >&2
  exit 3
fi
TORCH_DIR="$(python3 -c 'import torch, os; print(os.path.dirname(torch.__file__))')"
CXX="${CXX:-g++}"
mkdir -p "$OUT/obj"
FLAGS=(-std=c++17 -O2 -fPIC -w -D_GLIBCXX_USE_CXX11_ABI=1
       -include "$HERE/shim/prelude.h"
       -I "$HERE/shim" -I "$REF_SRC"
       -isystem "$TORCH_DIR/include" -isystem "$TORCH_DIR/include/torch/csrc/api/include")
SRCS=("$REF_SRC/Cloth.cpp" "$REF_SRC/PhysicsCloth.cpp" "$REF_SRC/MatrixMp.cpp" "$REF_SRC/Mesh.cpp"
      "$REF_SRC/Geometry.cpp" "$REF_SRC/BVH.cpp" "$REF_SRC/CollisionUtil.cpp" "$REF_SRC/Render.cpp"
      "$HERE/shim/eigen_cg.cpp"
      "$HERE/ref_harness.cpp")
pids=()
for s in "${SRCS[@]}"; do
  o="$OUT/obj/$(basename "${s%.cpp}").o"
  if [ ! -f "$o" ] || [ "$s" -nt "$o" ] || [ "$HERE/shim/prelude.h" -nt "$o" ]; then
    "$CXX" "${FLAGS[@]}" -c "$s" -o "$o" &
    pids+=($!)
  fi
done
for p in "${pids[@]}"; do wait "$p"; done
"$CXX" -o "$OUT/ref_harness" "$OUT"/obj/*.o \
  -L "$TORCH_DIR/lib" -Wl,-rpath,"$TORCH_DIR/lib" -ltorch -ltorch_cpu -lc10 -lgomp -lpthread
echo "built $OUT/ref_harness"
