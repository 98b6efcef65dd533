#!/usr/bin/env bash
# Builds the reference kfft library (SkyMaverick/kfft v0.8.1) straight from its
# C sources with gcc, for use as the parity oracle and the timed CPU baseline.
# It does not run the reference's own meson build; it writes a kfft_config.h
# equivalent to the README benchmark build (SYSMATH + OpenMP + Rader,
# RADER_LIMIT=25, PLAN_LEVEL=7, BFLY_LEVEL=5, extensions 2d/conv/conv2d) and
# compiles the listed translation units.  SIMD is left off: the reference's only
# SIMD path is x86 SSE, which the aarch64 hosts cannot build, so the portable C
# butterflies are used on every host for identical numerics.
#
# Usage: oracle/build_ref.sh [REFERENCE_SOURCE_DIR]
# Output: oracle/_ref/libkfft_ref.so (double) and oracle/_ref/libkfft_ref_f.so
#         (float, KFFT_HALF_SCALAR), plus oracle/_ref/libkfft_ref_default.so
#         (meson-default custom sqrt/sincos build, kept to document its defects).
set -euo pipefail
REF="${1:-/root/reference}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
mkdir -p "$OUT"
if [ ! -f "$REF/kfft.h" ]; then
    echo "build_ref.sh: reference sources not found at $REF" >&2
    exit 1
fi

write_cfg() {  # $1 = dir, $2 = extra defines (lines)
    mkdir -p "$1"
    cat > "$1/kfft_config.h" <<CFG
#pragma once
#define KFFT_MAJOR_VERSION 0
#define KFFT_MINOR_VERSION 8
#define KFFT_PATCH_VERSION 1
#define KFFT_DYNAPI_ENABLE
#define KFFT_USE_OPENMP
#define OMP_MINVER 201307
#define KFFT_RADER_ALGO
#define KFFT_RADER_LIMIT 25
#define KFFT_PLAN_LEVEL 7
#define KFFT_BFLY_LEVEL 5
#define KFFT_2D_ENABLE
#define KFFT_CONV_ENABLE
#define KFFT_CONV2_ENABLE
#define KFFT_CONV2D_ENABLE
$2
CFG
}

SRCS="kfft_pool.c kfft_cpx.c kfft_scalar.c kfft_ext.c kfft_math.c kfft_shift.c \
      ext/2d/kfft_cpx2.c ext/2d/kfft_scalar2.c ext/conv/kfft_cpx_conv.c \
      ext/conv/kfft_scalar_conv.c ext/conv2d/kfft_cpx_conv.c ext/conv2d/kfft_scalar_conv.c"

build() {  # $1 = name, $2 = cfg dir, $3 = extra sources
    local name="$1" cfg="$2" extra="$3"
    local objdir="$OUT/obj_$name"
    mkdir -p "$objdir"
    local objs=""
    for s in $SRCS $extra; do
        local o="$objdir/$(echo "$s" | tr '/' '_' | sed 's/\.c$/.o/')"
        gcc -std=gnu11 -O3 -ffast-math -funroll-loops -fPIC -fopenmp -DKFFT_EXPORTS \
            -I"$cfg" -I"$REF" -I"$REF/incs" -I"$REF/ext" -I"$REF/simd" -I"$REF/math" \
            -w -c "$REF/$s" -o "$o" &
        objs="$objs $o"
    done
    wait
    gcc -shared -fopenmp -o "$OUT/$name.so" $objs -lm
    rm -rf "$objdir"
}

write_cfg "$OUT/cfg_double" "#define KFFT_USE_SYSMATH"
write_cfg "$OUT/cfg_float" "#define KFFT_USE_SYSMATH
#define KFFT_HALF_SCALAR"
write_cfg "$OUT/cfg_default" "#undef KFFT_RADER_LIMIT
#define KFFT_RADER_LIMIT 11"

build libkfft_ref "$OUT/cfg_double" ""
build libkfft_ref_f "$OUT/cfg_float" ""
build libkfft_ref_default "$OUT/cfg_default" "math/kfft_scd.c"
uname -m > "$OUT/HOST_ARCH"
echo "built reference libraries in $OUT"
