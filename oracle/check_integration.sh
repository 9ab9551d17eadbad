#!/bin/sh
# Check the cellBP drop-in (wholecellfe_gb300/shim) against the reference (test
# infrastructure; nothing runs on a GPU):
#  1. UL_growth_gpu.cpp and cellbp_gpu_extras.cpp compile against the reference's headers
#     (kMD variant) and include/wcfe.h;
#  2. UL_growth_gpu.cpp links with a caller built from the reference's own declarations of
#     the mechanics functions (cellBP/main.cpp:72-87, read at check time) calling them as
#     main.cpp:224, :356 and :362-363 do, the reference's nondestructivetrimesh.cpp and
#     libwcfe.so.
# Writes only into oracle/_ref/shim.
#
# usage: oracle/check_integration.sh [REFERENCE_ROOT]   (default: $WCFE_REF or /root/reference)
# exit: 0 checked, 77 skipped (no reference sources or no libwcfe.so), else a failure
set -e
REF=${1:-${WCFE_REF:-/root/reference}}
HERE=$(cd "$(dirname "$0")" && pwd)
ROOT=$(cd "$HERE/.." && pwd)
SHIM="$ROOT/wholecellfe_gb300/shim"
OUT="$HERE/_ref/shim"
D="$REF/wholeCellFE_kMD"
if [ ! -d "$D/cellBP" ]; then
    echo "reference sources not found at $REF" >&2
    exit 77
fi
if [ ! -f "$ROOT/wholecellfe_gb300/libwcfe.so" ]; then
    echo "libwcfe.so not built" >&2
    exit 77
fi
mkdir -p "$OUT"
INC="-I$D/common -I$D/eltopo3d -I$D/cellBP -I$ROOT/include"
FLAGS="-std=c++17 -w -DNO_GUI -D__LITTLE_ENDIAN__"
g++ $FLAGS $INC -fsyntax-only "$SHIM/cellbp_gpu_extras.cpp"
{
    echo '#include "vec.h"'
    echo '#include "nondestructivetrimesh.h"'
    echo '#include <Eigen/Dense>'
    echo '#include <vector>'
    sed -n '72,87p' "$D/cellBP/main.cpp" | grep -E '^void (driverVelocities_Explicit|updateFA|updateForces_Explicit)\('
    cat <<'EOC'
void wcfe_gpu_attach(const NonDestructiveTriMesh& m, const std::vector<Vec3d>& x);
char g_output_path[256];
int main() {
    std::vector<Vec3d> X, x, V, Vh, A, fa;
    std::vector<Eigen::VectorXd> ea;
    std::vector<double> cA, cB, cC;
    NonDestructiveTriMesh m, ms;
    wcfe_gpu_attach(m, X);
    driverVelocities_Explicit(X, V, Vh, A, 1e-3);
    updateFA(cA, cC, fa, 1e-3, X, x, m, X, x, ms, -1.0);
    updateForces_Explicit(X, x, V, Vh, A, ea, cA, cB, cC, fa, 1e-3, 1e-3, m, 0.0);
    updateForces_Explicit(X, x, V, Vh, A, ea, 1e-3, 1e-3, ms, 0.0, fa, cC, x, m);
    return 0;
}
EOC
} > "$OUT/calls.cpp"
g++ $FLAGS $INC -c "$SHIM/UL_growth_gpu.cpp" -o "$OUT/shim.o"
g++ $FLAGS $INC -c "$OUT/calls.cpp" -o "$OUT/calls.o"
g++ $FLAGS $INC -c "$D/eltopo3d/nondestructivetrimesh.cpp" -o "$OUT/ndtm.o"
CUDA_LIB=${CUDA_HOME:-/usr/local/cuda}/lib64
g++ "$OUT/calls.o" "$OUT/shim.o" "$OUT/ndtm.o" -L"$ROOT/wholecellfe_gb300" -lwcfe -L"$CUDA_LIB" -lcudart \
    -o "$OUT/linked"
echo "integration shim: compiles and links"
