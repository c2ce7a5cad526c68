// Type-only stand-in for FastNoiseSIMD (an un-vendored, unpinned dependency of
// the reference).  It declares just enough for the reference's headers to
// compile; nothing here generates noise.  Test infrastructure only.
#pragma once
#include <cstdlib>
struct FastNoiseVectorSet {
  int size = 0;
  float* xSet = nullptr;
  float* ySet = nullptr;
  float* zSet = nullptr;
  int sampleScale = 0;
  int sampleSizeX = 0, sampleSizeY = 0, sampleSizeZ = 0;
  void SetSize(int n) {
    std::free(xSet);
    xSet = (float*)std::malloc(sizeof(float) * 3 * (size_t)(n > 0 ? n : 1));
    ySet = xSet + n; zSet = ySet + n; size = n;
  }
};
class FastNoiseSIMD {
 public:
  enum NoiseType { Value, ValueFractal, Perlin, PerlinFractal, Simplex, SimplexFractal, WhiteNoise, Cellular, Cubic, CubicFractal };
  enum FractalType { FBM, Billow, RigidMulti };
  enum PerturbType { None, Gradient, GradientFractal, Normalise, Gradient_Normalise, GradientFractal_Normalise };
  static FastNoiseSIMD* NewFastNoiseSIMD(int = 1337) { return new FastNoiseSIMD(); }
  static int GetSIMDLevel() { return 0; }
  static float* GetEmptySet(int x, int y, int z) { return (float*)std::malloc(sizeof(float) * (size_t)x * y * z); }
  void SetNoiseType(NoiseType) {}
  void SetFractalType(FractalType) {}
  void SetFractalOctaves(int) {}
  void SetFractalGain(float) {}
  void SetFractalLacunarity(float) {}
  void SetPerturbType(PerturbType) {}
  void SetPerturbFractalOctaves(int) {}
  void SetPerturbAmp(float) {}
  void SetPerturbFrequency(float) {}
  void SetPerturbFractalGain(float) {}
  void SetFrequency(float) {}
  void SetSeed(int) {}
  void FillNoiseSet(float*, FastNoiseVectorSet*, float = 0, float = 0, float = 0) {}
};
