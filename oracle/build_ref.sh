#!/usr/bin/env bash
# Test infrastructure only: builds the UNMODIFIED algorithms of the reference
# renderer (kennyalive/YAR, src/ref + src/lib + vendored pbrt-parser/pcg/
# tinyexr/stb) into oracle/_ref/ so that the oracle restatement in
# oracle/yar_oracle.c can be pinned against the reference's own output, and so
# that `bench.py --impl reference` can time the reference CPU path.
#
# The reference is an MSVC project; the edits below are portability-only
# (no algorithmic change): MSVC intrinsics -> GCC builtins, x86-only AES hash of
# the kd-tree cache directory name -> std::hash, MXCSR trap enabling -> no-op
# (exceptions stay masked, results are identical), and two extern/static
# mismatches.  Nothing here is committed: the patched copy lives in
# oracle/_ref/src (git-ignored) so it can be rebuilt on an aarch64 host that
# has no access to the reference tree.
#
# usage: oracle/build_ref.sh [REFERENCE_ROOT]
#   (default: $YAR_REFERENCE_ROOT, else a `reference` folder beside the repository)
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/_ref"
REF="${1:-${YAR_REFERENCE_ROOT:-$(cd "$HERE/../.." && pwd)/reference}}"
SRC="$OUT/src"

if [ -d "$REF/src/ref" ]; then
    rm -rf "$SRC"
    mkdir -p "$SRC/src" "$SRC/third-party"
    cp -r "$REF/src/lib" "$REF/src/ref" "$REF/src/std.h" "$REF/src/std.cpp" "$SRC/src/"
    for d in pbrt-parser pcg stb tinyexr tiny jsmn getopt; do
        cp -r "$REF/third-party/$d" "$SRC/third-party/"
    done
    chmod -R u+w "$SRC"
    C="$SRC/src/lib/common.h"
    sed -i 's/__debugbreak()/__builtin_trap()/' "$C"
    sed -i 's/^#error most_significant_bit_index.*/    return k ? 31u - (uint32_t)__builtin_clz(k) : 32u;/' "$C"
    sed -i 's/^#error allocate_aligned_memory.*/    return std::aligned_alloc(alignment, (size + alignment - 1) \/ alignment * alignment);/' "$C"
    sed -i 's/^#error free_aligned_memory.*/    std::free(ptr);/' "$C"
    sed -i 's/_mm_prefetch((const char\*)ptr, _MM_HINT_T0);/__builtin_prefetch(ptr);/' "$C"
    # count_leading_zeros: the non-MSVC branch has its own loop, keep it.
    CCPP="$SRC/src/lib/common.cpp"
    sed -i 's/^#include "immintrin.h"/#include <cstring>\n#include <iomanip>/' "$CCPP"
    sed -i 's/^#include "meow-hash\/meow_hash_x64_aesni.h"//' "$CCPP"
    sed -i 's/^    meow_u128 hash_128 = MeowHash(.*/    uint32_t hash_32 = (uint32_t)std::hash<std::string>{}(path_lowercase);/' "$CCPP"
    sed -i 's/^    uint32_t hash_32 = MeowU32From(hash_128, 0);//' "$CCPP"
    sed -i 's/__rdtsc()/0ull/g' "$CCPP"
    sed -i 's/^    _MM_SET_EXCEPTION_STATE(0);.*//; s/^    _MM_SET_EXCEPTION_MASK(.*//' "$CCPP"
    sed -i 's/\([^:a-z_]\)log2(/\1std::log2(/g' "$SRC/src/ref/shading_context.cpp"
    sed -i 's/end - BFIRST(ply)/end - (const char*)BFIRST(ply)/' "$SRC/third-party/pbrt-parser/impl/3rdParty/rply_reader.c"
fi
[ -d "$SRC/src/ref" ] || { echo "build_ref.sh: no reference sources (neither $REF nor $SRC)"; exit 2; }

mkdir -p "$OUT/obj"
CXX="${CXX:-g++}"
CCC="${CC:-gcc}"
CXXFLAGS="-O2 -std=c++20 -ffp-contract=off -fno-strict-aliasing -finput-charset=ISO-8859-1 -fpermissive -w -pthread \
 -include cstring -include cstdint -include cstdlib -include iomanip \
 -I$SRC/src -I$SRC/third-party -I$SRC/third-party/pbrt-parser/include -DNDEBUG"
LIB_SRCS=""
for f in "$SRC"/src/lib/*.cpp; do
    case "$(basename "$f")" in flying_camera.cpp) continue;; esac
    LIB_SRCS="$LIB_SRCS $f"
done
for f in "$SRC"/src/ref/*.cpp; do
    case "$(basename "$f")" in main.cpp|test*.cpp|benchmark*.cpp|intersection_simd.cpp) continue;; esac
    LIB_SRCS="$LIB_SRCS $f"
done
PBRT_SRCS="$(ls "$SRC"/third-party/pbrt-parser/impl/semantic/*.cpp "$SRC"/third-party/pbrt-parser/impl/syntactic/*.cpp)"

compile() {  # src -> obj name derived from path (the two Scene.cpp files differ by dir)
    local f="$1" o
    o="$OUT/obj/$(echo "${f#$SRC/}" | tr '/' '_' ).o"
    if [ ! -f "$o" ] || [ "$f" -nt "$o" ]; then
        $CXX $CXXFLAGS -c "$f" -o "$o"
    fi
}
export -f compile; export OUT SRC CXX CXXFLAGS
NPROC="$(nproc 2>/dev/null || echo 4)"
printf '%s\n' $LIB_SRCS $PBRT_SRCS | xargs -P "$NPROC" -I{} bash -c 'compile {}'
$CCC -O2 -w -c "$SRC/third-party/pbrt-parser/impl/3rdParty/rply_reader.c" -o "$OUT/obj/rply_reader.o"
$CCC -O2 -w -c "$SRC/third-party/pcg/pcg_basic.c" -o "$OUT/obj/pcg_basic.o"
rm -f "$OUT/libyarref.a"
ar rcs "$OUT/libyarref.a" "$OUT"/obj/*.o
$CXX $CXXFLAGS -I"$HERE" -I"$HERE/../include" -I"$HERE/../yar_gb300/csrc" "$HERE/ref_harness.cpp" "$OUT/libyarref.a" -o "$OUT/yar_ref" -pthread
echo "built $OUT/yar_ref"
# the drop-in render_scene_gpu: the reference's loader and builder, the product library's render
PRODUCT="$HERE/../yar_gb300/libyar_gb300.so"
if [ -f "$PRODUCT" ]; then
    $CXX $CXXFLAGS -I"$HERE" -I"$HERE/../include" -I"$HERE/../yar_gb300/csrc" "$HERE/render_scene_gpu.cpp" \
        "$OUT/libyarref.a" -L"$HERE/../yar_gb300" -lyar_gb300 -Wl,-rpath,'$ORIGIN/../../yar_gb300' \
        -o "$OUT/yar_ref_gpu" -pthread
    echo "built $OUT/yar_ref_gpu"
fi
