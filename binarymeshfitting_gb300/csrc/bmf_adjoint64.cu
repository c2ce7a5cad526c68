// The wide pass of the QEF adjoint (k_place_bwd<2, double | DF, 2>) in its own
// translation unit, built with FMA contraction: nothing here has to reproduce
// the reference's float rounding -- the branch of every listed vertex was
// decided by the exact FP32 replay of the first pass, and the FP32 eigenvectors
// only seed the refinement -- so the wide algebra may fuse multiplies and
// adds, and the double-float product needs fmaf.
#include "bmf_qef.cuh"

namespace bmf {

void launch_place_bwd_wide_list(int wide, const ChunkDev* d_chunks, int n_chunks, const uint32_t* words,
                                const float* dens, const uint32_t* vkey, const int64_t* d_counts, int64_t vcap,
                                const float* grad_pos, float* grad_dens, uint32_t* qlist, uint32_t* qcount,
                                float* qseed, cudaStream_t st) {
  const int blocks = (int)((vcap + 127) / 128);
  if (blocks == 0) return;
  if (wide == 2)
    k_place_bwd<2, DF, 2><<<blocks, 128, 0, st>>>(d_chunks, n_chunks, words, dens, vkey, d_counts, vcap, grad_pos,
                                                  grad_dens, qlist, qcount, qseed, nullptr);
  else
    k_place_bwd<2, double, 2><<<blocks, 128, 0, st>>>(d_chunks, n_chunks, words, dens, vkey, d_counts, vcap,
                                                      grad_pos, grad_dens, qlist, qcount, qseed, nullptr);
}

}  // namespace bmf
