#!/bin/bash
# Test infrastructure only: compile the reference combined_sieve from its own
# sources (read in place, never copied) against the declaration shims in
# oracle/refshim, into oracle/_ref/.  Three binaries are produced:
#   combined_sieve          unmodified sources
#   combined_sieve_wheelfix same sources with the inverted wheel test in
#                           combined_sieve.cpp:1134-1140 corrected, so jobs with
#                           gcd(d,210)=30 and SL > 30583 do not abort
#   gap_test_simple         unmodified sources (gap_test_simple.cpp,
#                           gap_test_common.cpp)
# Never built with -DNDEBUG: the reference has side effects inside assert().
# Needs the runtime libgmp.so.10 and libsqlite3.so.0; exits 0 with a message
# when the sources or libraries are absent.  The sources are read from
# PG_REFERENCE_DIR, by default the read-only mount of the build container
# (this recipe is the one file that names it).
set -eu
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${PG_REFERENCE_DIR:-/root/reference}"
OUT="$HERE/_ref"
mkdir -p "$OUT"

if [ ! -f "$REF/combined_sieve.cpp" ]; then
    echo "build_ref: reference sources not present, skipping"
    exit 0
fi

find_lib() {
    for d in /lib/x86_64-linux-gnu /usr/lib/x86_64-linux-gnu /lib/aarch64-linux-gnu \
             /usr/lib/aarch64-linux-gnu /usr/lib64 /usr/lib; do
        if [ -f "$d/$1" ]; then echo "$d/$1"; return 0; fi
    done
    return 1
}
GMP="$(find_lib libgmp.so.10 || true)"
SQL="$(find_lib libsqlite3.so.0 || true)"
if [ -z "$GMP" ] || [ -z "$SQL" ]; then
    echo "build_ref: libgmp.so.10 or libsqlite3.so.0 missing, skipping"
    exit 0
fi

CXXFLAGS="-O3 -fopenmp -std=c++17 -w -I$HERE/refshim -I$REF"
SRCS="$REF/gap_common.cpp $REF/modulo_search.cpp"

g++ $CXXFLAGS -o "$OUT/combined_sieve" "$REF/combined_sieve.cpp" $SRCS "$GMP" "$SQL"

# Wheel-fixed variant: the reference's own file piped through sed (not stored).
sed -e 's/if (wheel % 7) {/if (wheel % 7 == 0) {/' \
    -e 's/} else if (wheel % 5) {/} else if (wheel % 5 == 0) {/' \
    "$REF/combined_sieve.cpp" | \
    g++ $CXXFLAGS -o "$OUT/combined_sieve_wheelfix" -x c++ - -x none $SRCS "$GMP" "$SQL"

# The reference's CPU gap tester (mpz_probab_prime_p, mpz_prevprime/nextprime):
# the known answers of the probable-prime gap search.
g++ $CXXFLAGS -o "$OUT/gap_test_simple" "$REF/gap_test_simple.cpp" "$REF/gap_test_common.cpp" $SRCS "$GMP" "$SQL"

echo "build_ref: built $OUT/combined_sieve, $OUT/combined_sieve_wheelfix and $OUT/gap_test_simple"
