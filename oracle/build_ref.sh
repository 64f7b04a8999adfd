#!/bin/sh
# Recipe for the reference-literal oracle: compiles the reference's own
# lbm.cpp, unmodified and where it lies, against oracle/ref_config.h (which
# replaces the compile-time configuration block of LBM.h) and the Vector3d
# stand-in under oracle/shim, with the batch driver oracle/ref_harness.cpp.
# Outputs go to oracle/_ref/ only.  Needs the reference tree, given in the
# environment variable REF; without it this script does nothing and exits 0.
#
# usage: oracle/build_ref.sh [variant ...]
#   cavity:N[:TAU]            D3Q19 cavity, N^3 interior
#   details:N[:TAU]           the same cavity in MORE_DETAILS mode
#   cylinder:NX:NY:D:NODES:M  D2Q9 implicit IBM cylinder
#   explicit:NX:NY:D:NODES    the same cylinder, explicit direct forcing
#   transverse:NX:NY:D:NODES:M:AMP:FREQ  D2Q9 cylinder oscillating across the stream
#   sphere:NX:NY:NZ:D:RE:U    D3Q19 staircase sphere, momentum-exchange Cl/Cd
#   inline:NX:NY:D:NODES:M:PERIOD  D2Q9 cylinder oscillating along the stream (KC = 5)
#   arbie:NX:NY:D:NODES:M:CX  D2Q9 cylinder towed through fluid at rest
#   couette:NY:RE[:neumann]   D2Q9 thermal Couette flow (ENERGY: viscous heating, Dirichlet walls; the
#                             top wall a Neumann wall with j.n = 0)
#   poiseuille:NY:RE[:energy] D2Q9 body-forced channel (Poiseuille_Flow), optionally with ENERGY
#   cylbasic:NX:NY:D:RE:U     D2Q9 staircase cylinder, momentum-exchange Cl/Cd (Cylinder_Basic)
#   tandem:NX:NY:D:RE:U:LPD:NB    D2Q9 staircase circles in tandem (Cylinder_Tandem_Circle)
#   triangle:NX:NY:D:RE:U:LPD:NB  D2Q9 staircase triangles in tandem (Cylinder_Tandem_Triangle)
#   triangled:NX:NY:D:RE:U:LPD:NB the same in MORE_DETAILS mode
#   rayleigh:NX:NY:NZ         D3Q19 Rayleigh-Benard box (ENERGY, Dirichlet y walls, Neumann x and z walls)
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${REF:-}
OUT="$HERE/_ref"
if [ -z "$REF" ] || [ ! -f "$REF/lbm.cpp" ]; then
    echo "build_ref: no reference tree at $REF, skipped"
    exit 0
fi
mkdir -p "$OUT"
[ $# -eq 0 ] && set -- cavity:12:0.8 cavity:64:0.8 cylinder:80:40:10:40:5 sphere:48:24:24:8:20:0.05 details:8:0.8 \
    explicit:80:40:10:40 transverse:80:40:10:40:5:2.0:0.005 couette:30:20
CXX=${CXX:-g++}
FLAGS="-O2 -fopenmp -ffp-contract=off -w -include $HERE/ref_config.h -I$HERE/shim -I$REF"
pids=""
for v in "$@"; do
    kind=$(echo "$v" | cut -d: -f1)
    case "$kind" in
    cavity)
        n=$(echo "$v" | cut -d: -f2); tau=$(echo "$v" | cut -d: -f3); [ -z "$tau" ] && tau=0.8
        exe="$OUT/ref_cavity_${n}_${tau}"
        $CXX $FLAGS -DREF_CAVITY -DREF_NX=$n -DREF_NY=$n -DREF_NZ=$n -DREF_TAU=$tau \
            -o "$exe" "$REF/lbm.cpp" "$HERE/ref_harness.cpp" &
        pids="$pids $!" ;;
    details)
        n=$(echo "$v" | cut -d: -f2); tau=$(echo "$v" | cut -d: -f3); [ -z "$tau" ] && tau=0.8
        exe="$OUT/ref_details_${n}_${tau}"
        $CXX $FLAGS -DREF_CAVITY -DREF_DETAILS -DREF_NX=$n -DREF_NY=$n -DREF_NZ=$n -DREF_TAU=$tau \
            -o "$exe" "$REF/lbm.cpp" "$HERE/ref_harness.cpp" &
        pids="$pids $!" ;;
    cylinder)
        nx=$(echo "$v" | cut -d: -f2); ny=$(echo "$v" | cut -d: -f3); d=$(echo "$v" | cut -d: -f4)
        nodes=$(echo "$v" | cut -d: -f5); mm=$(echo "$v" | cut -d: -f6)
        exe="$OUT/ref_cylinder_${nx}_${ny}_${d}_${nodes}_${mm}"
        $CXX $FLAGS -DREF_CYLINDER -DREF_NX=$nx -DREF_NY=$ny -DREF_D=$d -DREF_NODES=$nodes -DREF_MMAX=$mm \
            -o "$exe" "$REF/lbm.cpp" "$HERE/ref_harness.cpp" &
        pids="$pids $!" ;;
    explicit)
        nx=$(echo "$v" | cut -d: -f2); ny=$(echo "$v" | cut -d: -f3); d=$(echo "$v" | cut -d: -f4)
        nodes=$(echo "$v" | cut -d: -f5)
        exe="$OUT/ref_explicit_${nx}_${ny}_${d}_${nodes}"
        $CXX $FLAGS -DREF_CYLINDER -DREF_EXPLICIT -DREF_NX=$nx -DREF_NY=$ny -DREF_D=$d -DREF_NODES=$nodes -DREF_MMAX=1 \
            -o "$exe" "$REF/lbm.cpp" "$HERE/ref_harness.cpp" &
        pids="$pids $!" ;;
    transverse)
        nx=$(echo "$v" | cut -d: -f2); ny=$(echo "$v" | cut -d: -f3); d=$(echo "$v" | cut -d: -f4)
        nodes=$(echo "$v" | cut -d: -f5); mm=$(echo "$v" | cut -d: -f6); amp=$(echo "$v" | cut -d: -f7)
        fr=$(echo "$v" | cut -d: -f8)
        exe="$OUT/ref_transverse_${nx}_${ny}_${d}_${nodes}_${mm}_${amp}_${fr}"
        $CXX $FLAGS -DREF_TRANSVERSE -DREF_NX=$nx -DREF_NY=$ny -DREF_D=$d -DREF_NODES=$nodes -DREF_MMAX=$mm \
            -DREF_AMP=$amp -DREF_FREQ=$fr -o "$exe" "$REF/lbm.cpp" "$HERE/ref_harness.cpp" &
        pids="$pids $!" ;;
    inline|arbie)
        kind=$(echo "$v" | cut -d: -f1)
        nx=$(echo "$v" | cut -d: -f2); ny=$(echo "$v" | cut -d: -f3); d=$(echo "$v" | cut -d: -f4)
        nodes=$(echo "$v" | cut -d: -f5); mm=$(echo "$v" | cut -d: -f6); p6=$(echo "$v" | cut -d: -f7)
        exe="$OUT/ref_${kind}_${nx}_${ny}_${d}_${nodes}_${mm}_${p6}"
        if [ "$kind" = inline ]; then extra="-DREF_INLINE -DREF_PERIOD=$p6"; else extra="-DREF_ARBIE -DREF_CX=$p6"; fi
        $CXX $FLAGS $extra -DREF_NX=$nx -DREF_NY=$ny -DREF_D=$d -DREF_NODES=$nodes -DREF_MMAX=$mm \
            -o "$exe" "$REF/lbm.cpp" "$HERE/ref_harness.cpp" &
        pids="$pids $!" ;;
    poiseuille)
        ny=$(echo "$v" | cut -d: -f2); re=$(echo "$v" | cut -d: -f3); en=$(echo "$v" | cut -d: -f4)
        exe="$OUT/ref_poiseuille_${ny}_${re}${en:+_energy}"
        $CXX $FLAGS -DREF_POISEUILLE ${en:+-DREF_ENERGY} -DREF_NY=$ny -DREF_RE=$re -o "$exe" "$REF/lbm.cpp" \
            "$HERE/ref_harness.cpp" &
        pids="$pids $!" ;;
    couette)
        ny=$(echo "$v" | cut -d: -f2); re=$(echo "$v" | cut -d: -f3); top=$(echo "$v" | cut -d: -f4)
        exe="$OUT/ref_couette_${ny}_${re}"; extra=""
        if [ "$top" = neumann ]; then exe="${exe}_neumann"; extra="-DREF_NEUMANN"; fi
        $CXX $FLAGS -DREF_COUETTE $extra -DREF_NY=$ny -DREF_RE=$re -o "$exe" "$REF/lbm.cpp" "$HERE/ref_harness.cpp" &
        pids="$pids $!" ;;
    cylbasic)
        nx=$(echo "$v" | cut -d: -f2); ny=$(echo "$v" | cut -d: -f3); d=$(echo "$v" | cut -d: -f4)
        re=$(echo "$v" | cut -d: -f5); u=$(echo "$v" | cut -d: -f6)
        exe="$OUT/ref_cylbasic_${nx}_${ny}_${d}_${re}_${u}"
        $CXX $FLAGS -DREF_CYLBASIC -DREF_NX=$nx -DREF_NY=$ny -DREF_D=$d -DREF_RE=$re -DREF_U=$u -o "$exe" \
            "$REF/lbm.cpp" "$HERE/ref_harness.cpp" &
        pids="$pids $!" ;;
    tandem|triangle|triangled)
        kind=$(echo "$v" | cut -d: -f1)
        nx=$(echo "$v" | cut -d: -f2); ny=$(echo "$v" | cut -d: -f3); d=$(echo "$v" | cut -d: -f4)
        re=$(echo "$v" | cut -d: -f5); u=$(echo "$v" | cut -d: -f6); lpd=$(echo "$v" | cut -d: -f7)
        nb=$(echo "$v" | cut -d: -f8)
        flag=-DREF_TANDEM; [ "$kind" = triangle ] && flag=-DREF_TRIANGLE
        [ "$kind" = triangled ] && flag="-DREF_TRIANGLE -DREF_DETAILS"
        exe="$OUT/ref_${kind}_${nx}_${ny}_${d}_${re}_${u}_${lpd}_${nb}"
        $CXX $FLAGS $flag -DREF_NX=$nx -DREF_NY=$ny -DREF_D=$d -DREF_RE=$re -DREF_U=$u -DREF_LPD=$lpd \
            -DREF_NB=$nb -o "$exe" "$REF/lbm.cpp" "$HERE/ref_harness.cpp" &
        pids="$pids $!" ;;
    rayleigh)
        nx=$(echo "$v" | cut -d: -f2); ny=$(echo "$v" | cut -d: -f3); nz=$(echo "$v" | cut -d: -f4)
        exe="$OUT/ref_rayleigh_${nx}_${ny}_${nz}"
        $CXX $FLAGS -DREF_RAYLEIGH -DREF_NX=$nx -DREF_NY=$ny -DREF_NZ=$nz -o "$exe" "$REF/lbm.cpp" \
            "$HERE/ref_harness.cpp" &
        pids="$pids $!" ;;
    sphere)
        nx=$(echo "$v" | cut -d: -f2); ny=$(echo "$v" | cut -d: -f3); nz=$(echo "$v" | cut -d: -f4)
        d=$(echo "$v" | cut -d: -f5); re=$(echo "$v" | cut -d: -f6); u=$(echo "$v" | cut -d: -f7)
        exe="$OUT/ref_sphere_${nx}_${ny}_${nz}_${d}_${re}_${u}"
        $CXX $FLAGS -DREF_SPHERE -DREF_NX=$nx -DREF_NY=$ny -DREF_NZ=$nz -DREF_D=$d -DREF_RE=$re -DREF_U=$u \
            -o "$exe" "$REF/lbm.cpp" "$HERE/ref_harness.cpp" &
        pids="$pids $!" ;;
    *) echo "unknown variant $v"; exit 2 ;;
    esac
done
for p in $pids; do wait $p; done
echo "build_ref: done -> $OUT"
