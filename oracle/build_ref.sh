#!/usr/bin/env bash
# Compiles the reference project's own CPU decoders (its pybind11 module
# `_native`, built from src/hsmm.cu + src/bindings.cpp with -DNO_GPU) straight
# from the read-only reference checkout into oracle/_ref/.  Nothing is copied
# into this repository: the sources are compiled where they lie.
#
# Four builds are produced:
#   oracle/_ref/shipped/_native*.so  the reference's own CPU flags
#                                    (CMakeLists.txt:131-136: -O3 -march=native
#                                    -mtune=native -ffast-math, OpenMP)
#   oracle/_ref/ieee/_native*.so     the same sources with plain IEEE
#                                    arithmetic (-O2, OpenMP, no fast-math), the
#                                    build the C restatement is pinned to
#   oracle/_ref/cuda/kernels_sm103a.cubin
#                                    the reference's CUDA kernels (src/kernels.cu)
#                                    for sm_103a with its CUDA flags
#                                    (CMakeLists.txt:141-148: -O3 -use_fast_math
#                                    -Xptxas=-O3), plus kernels.names, their
#                                    mangled names (nm of the host object).
#                                    Device code only: it runs on the GPU host
#                                    under oracle/ref_cuda.c, a host driver
#                                    written here that restates the reference's
#                                    launch sequence (src/hsmm.cu:604-791).
#   oracle/_ref/hsmmlearn/base*.so   hsmmlearn's compiled core (forward-backward
#                                    of the EM fit), see build_hsmmlearn below
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]
# The reference checkout is the argument, else $TV_REFERENCE_ROOT, else the
# development host's read-only checkout at /root/reference.  The root found is
# recorded in oracle/_ref/ROOT, where the tests and the fixture script look it
# up.  Exits 0 without building when the checkout or pybind11 is absent.
set -euo pipefail
REF="${1:-${TV_REFERENCE_ROOT:-/root/reference}}"
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/_ref"
if [[ ! -f "$REF/src/hsmm.cu" || ! -f "$REF/src/bindings.cpp" ]]; then
    echo "build_ref: reference sources not found under $REF; skipping" >&2
    exit 0
fi
mkdir -p "$OUT"
echo "$REF" > "$OUT/ROOT"
PY="${PYTHON:-python3}"
if ! PYBIND_INC="$($PY -c 'import pybind11; print(pybind11.get_include())' 2>/dev/null)"; then
    echo "build_ref: pybind11 not importable; skipping" >&2
    exit 0
fi
PY_INC="$($PY -c 'import sysconfig; print(sysconfig.get_path("include"))')"
SUFFIX="$($PY -c 'import sysconfig; print(sysconfig.get_config_var("EXT_SUFFIX"))')"

build() {
    local name="$1"; shift
    mkdir -p "$OUT/$name"
    local obj="$OUT/$name/_native$SUFFIX"
    if [[ -f "$obj" && "$obj" -nt "$REF/src/hsmm.cu" && "$obj" -nt "$REF/src/bindings.cpp" ]]; then
        return 0
    fi
    g++ -std=c++17 -shared -fPIC -DNO_GPU "$@" -fopenmp \
        -I"$REF/src" -isystem "$PY_INC" -isystem "$PYBIND_INC" \
        -x c++ "$REF/src/hsmm.cu" -x c++ "$REF/src/bindings.cpp" \
        -o "$obj.tmp"
    mv "$obj.tmp" "$obj"
    echo "build_ref: built $obj"
}

build_cuda() {
    local out="$OUT/cuda"
    local nv="${NVCC:-$(command -v nvcc || echo /usr/local/cuda/bin/nvcc)}"
    if [[ ! -x "$nv" ]]; then
        echo "build_ref: nvcc not found; the reference CUDA kernels are not built" >&2
        return 0
    fi
    mkdir -p "$out"
    if [[ -f "$out/kernels_sm103a.cubin" && "$out/kernels_sm103a.cubin" -nt "$REF/src/kernels.cu" \
          && -f "$out/kernels.names" ]]; then
        return 0
    fi
    local flags=(-gencode arch=compute_103a,code=sm_103a -O3 -use_fast_math -std=c++17 -I"$REF/src")
    "$nv" -cubin "${flags[@]}" -Xptxas=-O3 "$REF/src/kernels.cu" -o "$out/kernels_sm103a.cubin.tmp"
    "$nv" -c "${flags[@]}" "$REF/src/kernels.cu" -o "$out/kernels_host.o"
    # "<name> <mangled>" per kernel; the name is the mangled name's
    # length-prefixed identifier (_Z<len><name>...)
    nm "$out/kernels_host.o" | awk '$2 == "T" && $3 ~ /^_Z[0-9]+kernel_/ {
        s = substr($3, 3); match(s, /^[0-9]+/); len = substr(s, 1, RLENGTH) + 0;
        print substr(s, RLENGTH + 1, len), $3 }' > "$out/kernels.names.tmp"
    rm -f "$out/kernels_host.o"
    mv "$out/kernels_sm103a.cubin.tmp" "$out/kernels_sm103a.cubin"
    mv "$out/kernels.names.tmp" "$out/kernels.names"
    echo "build_ref: built $out/kernels_sm103a.cubin"
}

# The reference's training step: hsmmlearn's compiled core (its Cython
# wrapper base.pyx over _hsmm/src/*.cpp, the forward-backward of
# FBImpl.cpp), built as the Python extension oracle/_ref/hsmmlearn/base*.so
# with the package's own flags (setup.py: -fopenmp), so that its Python
# package under the checkout (hsmm.py's fit) can run against it.
build_hsmmlearn() {
    local out="$OUT/hsmmlearn"
    local src="$REF/hsmmlearn/hsmmlearn"
    if [[ ! -f "$src/base.pyx" ]]; then
        echo "build_ref: hsmmlearn sources not found; skipping" >&2
        return 0
    fi
    if ! "$PY" -c 'import Cython' 2>/dev/null; then
        echo "build_ref: Cython not importable; hsmmlearn not built" >&2
        return 0
    fi
    mkdir -p "$out"
    local so="$out/base$SUFFIX"
    if [[ -f "$so" && "$so" -nt "$src/base.pyx" && "$so" -nt "$src/_hsmm/src/FBImpl.cpp" ]]; then
        return 0
    fi
    "$PY" -m cython --cplus -3 -o "$out/base.cpp" "$src/base.pyx"
    g++ -O2 -fPIC -shared -fopenmp -isystem "$PY_INC" -I"$src" "$out/base.cpp" "$src"/_hsmm/src/*.cpp -o "$so.tmp"
    mv "$so.tmp" "$so"
    echo "build_ref: built $so"
}

build shipped -O3 -march=native -mtune=native -ffast-math &
build ieee -O2 &
build_cuda &
build_hsmmlearn &
wait
