#!/usr/bin/env bash
# Test infrastructure: compiles the reference's own operator sources, where
# they lie in the reference tree, into oracle/_ref/libsmilei_ref_ops.so.
#
# Only the files the hot path needs are compiled (interpolators, pushers,
# projectors, Yee solvers, fields, particles, radiation tables and the
# Monte-Carlo radiation operator), directly with
# g++; the reference's own build system is not used.  The reference headers
# name MPI and HDF5 types, so oracle/shims supplies declaration-level,
# single-rank stand-ins for <mpi.h> and <hdf5.h>; none of the compiled
# operators calls either library.  The result is loaded only by tests/ and by
# tests/golden/make_golden.py to pin the C restatement in oracle/pic_oracle.c.
#
# usage: oracle/build_ref.sh [reference_src_dir]
#   (default: $SMILEI_REFERENCE_SRC, else ../reference/src beside the checkout)
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
SRC="${1:-${SMILEI_REFERENCE_SRC:-$HERE/../../reference/src}}"
OUT="$HERE/_ref"
if [ ! -d "$SRC" ]; then
    echo "build_ref: reference sources not found at $SRC; skipping" >&2
    exit 0
fi
mkdir -p "$OUT/obj"

INC="-I$HERE/shims"
while IFS= read -r d; do INC="$INC -I$d"; done < <(find "$SRC" -type d)
INC="$INC $(python3-config --includes) -I$(python3 -c 'import numpy; print(numpy.get_include())')"
CXXFLAGS="-std=c++14 -O2 -fPIC -fopenmp -D__VERSION=\"ref\" -DOMPI_SKIP_MPICXX -D_OMP -w"

SOURCES="
Interpolator/Interpolator.cpp Interpolator/Interpolator2D.cpp Interpolator/Interpolator3D.cpp
Interpolator/Interpolator2D2Order.cpp Interpolator/Interpolator3D2Order.cpp
Pusher/Pusher.cpp Pusher/PusherBoris.cpp Pusher/PusherVay.cpp Pusher/PusherHigueraCary.cpp
Projector/Projector.cpp Projector/Projector2D.cpp Projector/Projector3D.cpp
Projector/Projector2D2Order.cpp Projector/Projector3D2Order.cpp
ElectroMagnSolver/MA_Solver2D_norm.cpp ElectroMagnSolver/MA_Solver3D_norm.cpp
ElectroMagnSolver/MF_Solver2D_Yee.cpp ElectroMagnSolver/MF_Solver3D_Yee.cpp
Field/Field.cpp Field/Field2D.cpp Field/Field3D.cpp Particles/Particles.cpp
Radiation/RadiationTables.cpp Radiation/RadiationTablesDefault.cpp Radiation/Radiation.cpp Radiation/RadiationMonteCarlo.cpp Radiation/Table.cpp Radiation/Table2D.cpp
SmileiMPI/AsyncMPIbuffers.cpp Tools/H5.cpp Particles/Particle.cpp
ElectroMagnBC/ElectroMagnBC.cpp ElectroMagnBC/ElectroMagnBC2D.cpp ElectroMagnBC/ElectroMagnBC2D_SM.cpp
ElectroMagn/Laser.cpp Profiles/Function.cpp Profiles/Profile.cpp Tools/gpu.cpp
"

pids=()
objs=()
for s in $SOURCES; do
    o="$OUT/obj/$(basename "$s" .cpp).o"
    objs+=("$o")
    if [ ! -f "$o" ] || [ "$SRC/$s" -nt "$o" ]; then
        g++ $CXXFLAGS $INC -c "$SRC/$s" -o "$o" &
        pids+=($!)
    fi
done
o="$OUT/obj/ref_driver.o"
objs+=("$o")
g++ $CXXFLAGS $INC -c "$HERE/ref_driver.cpp" -o "$o" &
pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done

# Functions the compiled operators reference but never call on this path
# (namelist parsing, diagnostics, MPI exchange) stay undefined and are bound
# lazily; the library is only ever loaded by the test harness.
g++ -shared -fopenmp -o "$OUT/libsmilei_ref_ops.so" "${objs[@]}" -Wl,--allow-shlib-undefined
echo "build_ref: $OUT/libsmilei_ref_ops.so"

# The reference's own CUDA current deposits (Projector{3D,2D}2OrderGPUKernelCUDAHIP.cu,
# the kernels its NVIDIA builds launch from Projector{3D,2D}2OrderGPU) as device code
# only: cubins for sm_103a, loaded through the driver API by oracle/ref_gpu_deposit.py on a GPU
# host to time it beside this project's kernel.  The defines are those of the
# reference's OpenACC + CUDA build; its host code is not used.
NVCC="${NVCC:-/usr/local/cuda/bin/nvcc}"
if [ -x "$NVCC" ]; then
    for D in 3 2; do
        if "$NVCC" -cubin -gencode arch=compute_103a,code=sm_103a -std=c++14 -O3 --expt-relaxed-constexpr \
            -DSMILEI_ACCELERATOR_GPU -DSMILEI_ACCELERATOR_GPU_OACC -D__VERSION=\"ref\" -DOMPI_SKIP_MPICXX -w $INC \
            -Xptxas -v "$SRC/Projector/Projector${D}D2OrderGPUKernelCUDAHIP.cu" -o "$OUT/ref_deposit${D}d.cubin" \
            > "$OUT/ref_deposit${D}d.ptxas.txt" 2>&1; then
            # the current deposit's entry name, as ptxas reports it
            grep -o "_ZN[0-9]*cudahip[0-9a-z]*6kernel31DepositCurrentDensity_${D}D_Order2[A-Za-z0-9_]*" \
                "$OUT/ref_deposit${D}d.ptxas.txt" | head -1 > "$OUT/ref_deposit${D}d.entry"
            echo "build_ref: $OUT/ref_deposit${D}d.cubin"
        else
            echo "build_ref: the reference's ${D}D CUDA deposit did not compile (see $OUT/ref_deposit${D}d.ptxas.txt)" >&2
        fi
    done
fi
