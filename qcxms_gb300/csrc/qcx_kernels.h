// Kernel launchers shared between the translation units of libqcxgpu.
#pragma once
#include <cuda_runtime.h>

#include "qcx_batch.cuh"

namespace qcx {

void launch_cn(const DevBatch& bt, cudaStream_t st);
// The shell-pair kernels launch one specialised kernel per angular-momentum
// class; they return the number of kernels launched.
int launch_integrals(const DevBatch& bt, cudaStream_t st);
void launch_scc(const DevBatch& bt, int precision, cudaStream_t st);
int launch_grad_pairs(const DevBatch& bt, cudaStream_t st);
void launch_grad_atoms(const DevBatch& bt, cudaStream_t st);
void launch_leapfrog(const DevBatch& bt, double tstep, cudaStream_t st);
void launch_zero_grad(const DevBatch& bt, cudaStream_t st);
// fragment numbers of every molecule's atoms (frag[natom]) and fragment counts (nfrag[nmol])
void launch_fragments(const DevBatch& bt, int max_nat, const double* rad, double rcut, int at1, int at2, int* frag,
                      int* nfrag, cudaStream_t st);

// dynamic shared memory the SCC kernel asks for, given the largest molecule
size_t scc_smem_bytes(int max_nao, int precision);

}  // namespace qcx
