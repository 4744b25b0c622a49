#!/bin/bash
# Builds the reference M-THEMES `forge` from its sources where they lie
# (the directory named by MTH_REFERENCE, required) into oracle/_ref/ only,
# for pinning the oracle.  It compiles the reference's own 8 translation units
# (src/Makefile:11) with single-rank MPI/FFTW-MPI/GSL stand-ins
# (oracle/refshim) and serial FFTW 2.1.5 built from the vendored tarball.
# The reference's build system and MPICH are not used.  x86 or Arm host; no
# GPU needed.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${MTH_REFERENCE:?set MTH_REFERENCE to the reference checkout}"
OUT="$HERE/_ref"
if [ ! -d "$REF/src" ]; then echo "reference sources not found at $REF" >&2; exit 2; fi
mkdir -p "$OUT/obj"
if [ ! -f "$OUT/fftw/lib/libfftw.a" ]; then
  rm -rf "$OUT/fftw-src"; mkdir -p "$OUT/fftw-src"
  tar xzf "$REF/fftw/src/fftw-2.1.5.tar.gz" -C "$OUT/fftw-src"
  ( cd "$OUT/fftw-src/fftw-2.1.5" && \
    ./configure --prefix="$OUT/fftw" --disable-shared CFLAGS="-O2 -fPIC" > ../configure.log 2>&1 && \
    make -j8 > ../make.log 2>&1 && make install > ../install.log 2>&1 )
fi
CXX="${CXX:-g++}"
COMMON=(-O3 -w -fPIC -include "$HERE/refshim/mth_ref_prelude.h" -I"$HERE/refshim" -I"$OUT/fftw/include" -I"$REF/src")
declare -A EXTRA
EXTRA[evp.c]="-DSetupJob=mth_ref_SetupJob -DDestroyJob=mth_ref_DestroyJob"
EXTRA[evolution.c]="-DStrainRate_Orowan=StrainRate_eval -DDislocationEvolution=mth_ref_after_step -DAvgDislocation=mth_ref_noop -DGradient_ShearRate=mth_ref_noop -DGradient_Shear=mth_ref_noop -DVonMises=mth_ref_VonMises"
OBJS=()
for s in evp.c io.c init.c kinematics.c evolution.c constitutive.c integrated.c pf_xrx.c; do
  o="$OUT/obj/${s%.c}.o"
  # shellcheck disable=SC2086
  $CXX -x c++ "${COMMON[@]}" ${EXTRA[$s]:-} -c "$REF/src/$s" -o "$o" &
  OBJS+=("$o")
done
$CXX "${COMMON[@]}" -c "$HERE/refshim/refshim.cc" -o "$OUT/obj/refshim.o" &
# the shipped dislocation-density path: evolution.c with only the trace hooks
$CXX -x c++ "${COMMON[@]}" -DAvgDislocation=mth_ref_dd_after_step -DVonMises=mth_ref_VonMises \
  -c "$REF/src/evolution.c" -o "$OUT/obj/evolution_dd.o" &
# and with DD_CU as src/evpFlags.h ships it (fixed Cu elastic constants,
# src/init.c:821-825), for runs on the unmodified test_run/ inputs
$CXX -x c++ "${COMMON[@]}" -DDD_CU -c "$REF/src/init.c" -o "$OUT/obj/init_ddcu.o" &
# the DRX harness: PF_XRX with the per-substep grid hook of mth_ref_prelude.h,
# and evp.c without its main() for the global definitions
$CXX -x c++ "${COMMON[@]}" -DMTH_PF_HOOK -c "$REF/src/pf_xrx.c" -o "$OUT/obj/pf_xrx_hook.o" &
$CXX -x c++ "${COMMON[@]}" ${EXTRA[evp.c]} -Dmain=mth_ref_evp_main -c "$REF/src/evp.c" -o "$OUT/obj/evp_nomain.o" &
$CXX "${COMMON[@]}" -DMTH_PF_HOOK -c "$HERE/refshim/drx_harness.cc" -o "$OUT/obj/drx_harness.o" &
wait
$CXX -o "$OUT/forge_ref" "${OBJS[@]}" "$OUT/obj/refshim.o" -L"$OUT/fftw/lib" -lfftw -lm
DD_OBJS=("${OBJS[@]/evolution.o/evolution_dd.o}")
$CXX -o "$OUT/forge_ref_dd" "${DD_OBJS[@]}" "$OUT/obj/refshim.o" -L"$OUT/fftw/lib" -lfftw -lm
DDCU_OBJS=("${DD_OBJS[@]/init.o/init_ddcu.o}")
$CXX -o "$OUT/forge_ref_dd_cu" "${DDCU_OBJS[@]}" "$OUT/obj/refshim.o" -L"$OUT/fftw/lib" -lfftw -lm
H_OBJS=("${OBJS[@]/evp.o/evp_nomain.o}")
H_OBJS=("${H_OBJS[@]/pf_xrx.o/pf_xrx_hook.o}")
$CXX -o "$OUT/drx_ref" "${H_OBJS[@]}" "$OUT/obj/refshim.o" "$OUT/obj/drx_harness.o" -L"$OUT/fftw/lib" -lfftw -lm
echo "built $OUT/forge_ref $OUT/forge_ref_dd $OUT/forge_ref_dd_cu $OUT/drx_ref"
