/*
 * pnamp_gcm.h -- batched Hill-Wheeler (GCM) solves on the GPU (GB300, sm_103a).
 *
 * The consumer of the projected kernels: HNDIAG (Codes/GCM/GCM_HNDiag.f90:2-103)
 * diagonalises the norm matrix, keeps the natural states whose eigenvalue is at least
 * eps times the largest (the driver's cutoff eps = 1e-5, Codes/exec/GCM.sh:59), and
 * diagonalises N^-1/2 H N^-1/2 in that subspace. This entry point does the same for a
 * batch of independent problems (one per angular momentum of a GCM basis, and the
 * K-mixing of each vacuum alone), one CTA per problem, both eigenproblems by cyclic
 * complex Jacobi rotations in FP64.
 *
 * Matrices are row-major complex (interleaved re, im doubles), Hermitian (only what the
 * Hermitian part implies is used: (A + A^+)/2). All pointers are DEVICE pointers except
 * `dim` and `off`, which are host arrays. `stream` is a cudaStream_t (NULL = legacy
 * default stream). Return codes: 0 ok, 1 invalid argument, 2 CUDA error.
 */
#ifndef PNAMP_GCM_H
#define PNAMP_GCM_H

#ifdef __cplusplus
extern "C" {
#endif

#define PNAMP_HW_MAX_DIM 1024

/* Bytes of device work space pnamp_hw_solve needs for these problem sizes. */
long long pnamp_hw_work_bytes(int nprob, const int *dim);

/* Problem b has size dim[b] (1 .. PNAMP_HW_MAX_DIM); its matrices start at complex
 * element off[b] of H and N, and its outputs at off[b] of E (dim[b] doubles: the energies
 * in ascending order, the first kept[b] valid, the rest 0) and of F (optional, NULL for
 * none: dim[b] x dim[b] complex, column k = the k-th solution f_k in the original basis,
 * normalised f_k^+ N f_k = 1; columns >= kept[b] are 0). kept[b] = number of natural
 * states kept (0 when N has no positive eigenvalue). `work`: pnamp_hw_work_bytes bytes. */
int pnamp_hw_solve(int nprob, const int *dim, const long long *off, const double *H,
                   const double *N, double eps, double *E, int *kept, double *F, void *work,
                   void *stream);

#ifdef __cplusplus
}
#endif
#endif /* PNAMP_GCM_H */
