// process_gpu_1 for an unmodified gEpiCount, backed by libgepi.so.
//
// gEpiCount's main (src/gEpiCount.cpp:87) calls
//     void process_gpu_1(PlinkReader<ui8> *pr, InteractionResult *tops,
//                        const struct _paramP1 &par);
// declared at src/proc_gpu.h:134 and defined at src/kernels/kernel1.cu:508-511,
// and its printing calls the C function fisher_pval (inc/gEpiCount.h:137-139,
// src/misc/fisher_p.c:52-76).  This file defines both against the reference's
// own headers, so a maintainer links it (and libgepi.so) in place of
// kernel1.cu, misc1.cu, entropyD.cu, fisher_d.cu and fisher_p.c and keeps
// main, the reader, the QC report and the printing unchanged:
//
//     make -C integration REF=<gEpiCount tree>     (links integration/_build/gEpiCount)
//
// Inputs are read through the reader exactly as the reference's launcher reads
// them (BitData, ValidData, numSNPs, elementsSNP, classData(1|2)->mask()); the
// caller's zeroed tops[par.topmost] are filled ascending.  Errors are printed
// in the reference's CUDACHECK format and leave tops as they were (zeroed),
// as the reference leaves them after a failed CUDA call.
#include <cstdio>

#include "../inc/gEpiCount.h"
#include "gepi.h"

// The result records are written straight into the caller's array.
static_assert(sizeof(InteractionResult) == sizeof(gepi_result), "InteractionResult layout");
static_assert(offsetof(InteractionResult, sA) == offsetof(gepi_result, sA), "sA");
static_assert(offsetof(InteractionResult, sB) == offsetof(gepi_result, sB), "sB");
static_assert(offsetof(InteractionResult, n) == offsetof(gepi_result, n), "n");
static_assert(offsetof(InteractionResult, ent) == offsetof(gepi_result, ent), "ent");
static_assert(offsetof(InteractionResult, fun) == offsetof(gepi_result, fun), "fun");
static_assert(sizeof(ui8) == sizeof(uint64_t), "ui8 rows are 64-bit words");
static_assert((int)FFUNC_ENTROPY == GEPI_ENTROPY && (int)FFUNC_FISHERPV == GEPI_FISHER,
              "objective values");
static_assert((int)BFUNC_AND == GEPI_AND && (int)BFUNC_XOR == GEPI_XOR, "function values");

void process_gpu_1(PlinkReader<ui8> *pr, InteractionResult *tops, const struct _paramP1 &par) {
    SampleClassInfo<ui8> *c0 = pr->classData(1), *c1 = pr->classData(2);
    if (c0 == NULL || c1 == NULL || c0->mask() == NULL || c1->mask() == NULL) {
        std::fprintf(stderr, "Error in class mask data\n");
        return;
    }
    gepi_params gp = {};
    gp.gpu_num = par.gpuNum;
    gp.topmost = par.topmost;
    gp.objective = par.ffun == FFUNC_FISHERPV ? GEPI_FISHER : GEPI_ENTROPY;
    gp.method = GEPI_METHOD_AUTO;
    const gepi_status s = gepi_process_gpu_1(
        reinterpret_cast<const uint64_t *>(pr->BitData()),
        reinterpret_cast<const uint64_t *>(pr->ValidData()), (int)pr->numSNPs(),
        (int)pr->elementsSNP(), reinterpret_cast<const uint64_t *>(c0->mask()),
        reinterpret_cast<const uint64_t *>(c1->mask()), reinterpret_cast<gepi_result *>(tops), &gp);
    if (s != GEPI_OK)
        std::fprintf(stderr, "E[%d]: Error in process_gpu_1 (gepi): (%d) %s: %s\n", par.gpuNum,
                     (int)s, gepi_status_string(s), gepi_last_error());
}

// The 32-bit-element reader has no GPU path in the reference either
// (src/kernels/kernel1.cu:513-516 leaves it empty).
void process_gpu_1(PlinkReader<ui4> *pr, InteractionResult *tops, const struct _paramP1 &par) {
    (void)pr;
    (void)tops;
    std::fprintf(stderr, "E[%d]: process_gpu_1: 32-bit elements are not supported\n", par.gpuNum);
}

extern "C" float fisher_pval(int n11, int n12, int n21, int n22) {
    return gepi_fisher_pval(n11, n12, n21, n22);
}
