#!/usr/bin/env bash
# build_ref.sh -- compile the reference's own hot-path source for the pinning
# tests and the reference leg of bench.py (TEST INFRASTRUCTURE).
#
# Where the reference tree is present (REF_DIR; by default a directory named
# `reference` beside this repository's root) the
# needed source is cut from it into oracle/_ref/src (git-ignored) and patched
# at its undefined-behaviour sites only, with the defined meanings D1-D6
# listed in oracle/swm_oracle.c. Where it is absent (a machine that only
# received oracle/_ref/src) the same sources are compiled again from there.
# Outputs go to oracle/_ref/ only.
#   serial_index_verbatim  serial_index.c exactly as written (x86 shifts)
#   serial_index           serial_index.c with D1 + D2
#   libswref.so            mapper_cpe.c:78-133,214-660,1244-2590 with D1,D4,D6,
#                          DMA as memcpy and faaw as an atomic fetch-add
#   libswref_sam.so        mapper_mpe.c:31-69,315-687 (the SAM writer) with
#                          gzwrite / gzprintf appending to a memory buffer
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF_DIR="${REF_DIR:-$(cd "$HERE/../.." && pwd)/reference}"
OUT="$HERE/_ref"
SRC="$OUT/src"
SHIM="$HERE/ref_shim"
CC="${CC:-gcc}"
mkdir -p "$SRC"

if [ -f "$REF_DIR/serial_index.c" ] && [ -f "$REF_DIR/mapper_cpe.c" ]; then
  cp "$REF_DIR/serial_index.c" "$SRC/serial_index_verbatim.c"
  cp "$REF_DIR/kseq.h" "$REF_DIR/fm_define.h" "$SRC/"
  # D1 (funnel shift at s == 0) and D2 (guarded final flush, serial_index.c:423-426)
  sed -e 's/<< *( *32 *- *\([a-z_%0-9]*\))/<< ((32 - \1) \& 31) \& ZMASK(32 - \1)/g' \
      -e 's/<< ((16 - pos%16) \* 2)/<< (((16 - pos%16) * 2) \& 31) \& ZMASK((16 - pos%16) * 2)/' \
      -e '423,425s/^/    if (position % 32) /' \
      -e '426s/^/    if (position % 16) /' \
      "$REF_DIR/serial_index.c" > "$SRC/serial_index_defined.c"
  # mapper: types/macros, align_reads + scalar Myers, seeds .. get_positions
  { sed -n '78,133p' "$REF_DIR/mapper_cpe.c"
    sed -n '214,660p' "$REF_DIR/mapper_cpe.c"
    sed -n '1244,2590p' "$REF_DIR/mapper_cpe.c"; } |
  sed -e 's/<< *( *32 *- *\([a-z_]*\))/<< ((32 - \1) \& 31) \& ZMASK(32 - \1)/g' \
      -e 's/asm volatile("memb\\n\\t");//' \
      -e 's/asm volatile("faaw %0, 0(%1)\\n\\t":"=r"(\([a-z_]*\)):"r"((\([a-z_>-]*\))));/\1 = __atomic_fetch_add(\2, 1, __ATOMIC_RELAXED);/' \
      -e 's/(d0_arry_64\[i\]>>search_site)&mask_1/TBBIT(d0_arry_64[i], search_site)/g' \
      -e 's/(hp_arry_64\[i\]>>search_site)&mask_1/TBBIT(hp_arry_64[i], search_site)/g' \
      -e 's/if(sum_err==err) break;/if(sum_err==err) break; if(match_site < 0) break;/' \
      -e 's/^\( *\)sindex_t pre_small = invalid_value;/\1if (heap_size == 0) { pos_ind[0] = 0; return 1; }\n\1sindex_t pre_small = invalid_value;/' \
      > "$SRC/mapper_ref.c"
  # SAM writer: tags and formatting constants, sam_header .. sam_format_2
  { sed -n '31,69p' "$REF_DIR/mapper_mpe.c"
    sed -n '315,687p' "$REF_DIR/mapper_mpe.c"; } > "$SRC/sam_ref.c"
fi

if [ ! -f "$SRC/mapper_ref.c" ]; then
  echo "build_ref: no reference source available" >&2
  exit 2
fi

# -fsigned-char: the reference prints CIGAR run lengths as '0' + (char)v % 10
# (mapper_cpe.c:223), which depends on char being signed; it is pinned as
# built on x86, where it is. Arm's default unsigned char would print other
# bytes for runs of 128 or more.
CFLAGS="-O2 -std=gnu99 -fgnu89-inline -fsigned-char -w"
$CC $CFLAGS -I"$SHIM" -I"$SRC" "$SRC/serial_index_verbatim.c" -Wl,--wrap=malloc -o "$OUT/serial_index_verbatim"
$CC $CFLAGS -I"$SHIM" -I"$SRC" -include "$SHIM/ub_defined.h" "$SRC/serial_index_defined.c" -Wl,--wrap=malloc -o "$OUT/serial_index"
$CC $CFLAGS -fPIC -ftrivial-auto-var-init=zero -I"$SHIM" -I"$SRC" -include "$SHIM/mapper_prelude.h" \
    -c "$SRC/mapper_ref.c" -o "$OUT/mapper_ref.o"
$CC $CFLAGS -fPIC -I"$SHIM" -I"$SRC" -c "$SHIM/mapper_driver.c" -o "$OUT/mapper_driver.o"
$CC -shared -o "$OUT/libswref.so" "$OUT/mapper_ref.o" "$OUT/mapper_driver.o" -lpthread
if [ -f "$SRC/sam_ref.c" ]; then
  $CC $CFLAGS -fPIC -I"$SHIM" -I"$SRC" -include "$SHIM/sam_prelude.h" -c "$SRC/sam_ref.c" -o "$OUT/sam_ref.o"
  $CC $CFLAGS -fPIC -I"$SHIM" -I"$SRC" -c "$SHIM/sam_driver.c" -o "$OUT/sam_driver.o"
  $CC -shared -o "$OUT/libswref_sam.so" "$OUT/sam_ref.o" "$OUT/sam_driver.o"
fi
echo "build_ref: ok"
