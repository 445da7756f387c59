/*
 * Device code of the reference's own CUDA kernels, for the GPU machine (TEST
 * INFRASTRUCTURE ONLY).  oracle/build_ref.sh compiles this file with the
 * reference's cuda/periodicBrinkman.h, where the reference tree exists, into
 * a device-only image (oracle/_ref/ref_kernels.cubin, plus a PTX copy the
 * driver can compile where the cubin is not accepted).  The image holds
 * kernelReal and kernelFourier (cuda/periodicBrinkman.h:219-425) exactly as
 * the reference wrote them; oracle/ref_launch.cpp loads it through the CUDA
 * driver API and launches them as the reference's periodicBrinkman() does
 * (cuda/periodicBrinkman.h:432-513).  The reference's sources never enter
 * this repository; only the compiled image travels.
 */
#include "periodicBrinkman.h"
