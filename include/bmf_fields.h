/* Density-field identifiers and parameter layouts shared by the C ABI
 * (include/bmf.h), the CUDA kernels and the CPU oracle.
 *
 * A field is evaluated at world position p = origin + (x, y, z) * scale for
 * sample (x, y, z) of a chunk, exactly as the reference's block samplers build
 * their coordinates (ImplicitSampler.hpp:22-33: dxyz.x = p.x + (float)x * scale).
 * A sample is "inside" when its value is < 0 (DMCChunk.cpp:136).
 */
#ifndef BMF_FIELDS_H
#define BMF_FIELDS_H

/* Caller-supplied density grid (no evaluation; the Sampler::block plugin case). */
#define BMF_FIELD_GRID 0
/* |p - c| - r + a * sin(k x) sin(k y) sin(k z)
 * params: [0..2] centre c, [3] radius r, [4] amplitude a, [5] wave number k.
 * sin is this project's own Cody-Waite + Taylor evaluation, bit-identical on
 * the GPU and in the oracle. */
#define BMF_FIELD_SPHERE_WAVE 1
/* (y - h) - a * FBM(p), FBM = sum over octaves o of gain^o * perlin(p * freq * lacunarity^o)
 * with K. Perlin's improved gradient noise (SIGGRAPH 2002).
 * params: [0] h, [1] a, [2] freq, [3] lacunarity, [4] gain, [5] octaves,
 * [6] seed (integer-valued).  The permutation is a Fisher-Yates shuffle of
 * 0..255 driven by splitmix64(seed). */
#define BMF_FIELD_TERRAIN_FBM 2
/* The reference's analytic fields (ImplicitSampler.cpp:27-65); params[0] is
 * the sampler's world_size ("resolution"). */
#define BMF_FIELD_TORUS_Z 3
#define BMF_FIELD_SPHERE 4
#define BMF_FIELD_CUBOID 5
#define BMF_FIELD_PLANE_Y 6
/* The shape of the reference's default world sampler, a 2D heightmap with a
 * perturbed domain (NoiseSamplers::terrain2d_pert_block, NoiseSampler.cpp:148-194,
 * selected at WorldOctree.cpp:40): density = -(y * g) - height * n(x, z), with
 * n a value-noise FBM over a gradient-noise-perturbed (x, z).  The reference
 * draws both noises from FastNoiseSIMD (not vendored); this project restates
 * them (2D value noise with quintic fade, 2D gradient noise with 8 directions),
 * evaluated identically by the GPU and the oracle:
 *   (xn, zn) = (x * g, z * g) * 0.01;
 *   per perturb octave k < pert_octaves (frequency f_k = pert_freq * 2^k,
 *   amplitude a_k = pert_amp * pert_gain^k), with (sx, sz) = (xn, zn) * f_k
 *   taken before the octave:
 *     xn += a_k * grad2_0(sx, sz),  zn += a_k * grad2_1(sx, sz);
 *   n = sum_o 0.5^o value2(xn * 2^o, zn * 2^o) / sum_o 0.5^o over value_octaves.
 * params: [0] g (g_scale), [1] height, [2] pert_octaves, [3] pert_amp,
 * [4] pert_freq, [5] pert_gain, [6] seed (integer-valued, as BMF_FIELD_TERRAIN_FBM),
 * [7] value_octaves.  WorldOctree.cpp:49-55 uses g 0.25, height 75, 13 octaves,
 * amp 0.87, freq 0.585, gain 0.488 (FastNoiseSIMD's default FBM has 3 octaves). */
#define BMF_FIELD_TERRAIN_2D 7

#define BMF_FIELD_MAX_PARAMS 8

#endif
