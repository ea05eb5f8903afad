// Driver linked with the reference's LinearScan/randomVectorGenerator.cpp (compiled from
// the read-only reference tree into oracle/_ref/) to dump its host random streams as
// golden vectors.  Usage: rng_driver <kind> <count> [sketchDim] > out.bin
//   kind 0: generateRandomVectors(float*, N)          N(0,1)   (randomVectorGenerator.cpp:32-53)
//   kind 1: generateRandomVectors(N, sketchDim)       N(0,1/s) (randomVectorGenerator.cpp:56-74)
//   kind 2: generateRandomOnePlusMinusVector(N, int*)          (randomVectorGenerator.cpp:76-87)
//   kind 3: the call weightedMinHash.cuh:231-250 makes (uniform_int(0,1) bools)
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>
#include <unistd.h>

float* generateRandomVectors(int N, bool randomSeed = false);
float* generateRandomVectors(int N, int sketchDim, bool randomSeed = false);
void generateRandomVectors(float* vectors, int N, bool randomSeed = false);
void generateRandomOnePlusMinusVector(int size, int* vectors);

int main(int argc, char** argv) {
  if (argc < 3) return 2;
  int kind = atoi(argv[1]), n = atoi(argv[2]);
  // the reference prints progress on stdout: keep stdout for the binary payload
  int saved = dup(1);
  freopen("/dev/null", "w", stdout);
  std::vector<unsigned char> out;
  if (kind == 0) {
    std::vector<float> v(n);
    generateRandomVectors(v.data(), n);
    out.assign((unsigned char*)v.data(), (unsigned char*)(v.data() + n));
  } else if (kind == 1) {
    float* v = generateRandomVectors(n, atoi(argv[3]));
    out.assign((unsigned char*)v, (unsigned char*)(v + n));
  } else if (kind == 2) {
    std::vector<int> v(n);
    generateRandomOnePlusMinusVector(n, v.data());
    out.assign((unsigned char*)v.data(), (unsigned char*)(v.data() + n));
  } else {
    std::default_random_engine generator;
    std::uniform_int_distribution<int> distribution(0, 1);
    for (int i = 0; i < n; ++i) out.push_back((unsigned char)(distribution(generator) != 0));
  }
  fflush(stdout);
  dup2(saved, 1);
  fwrite(out.data(), 1, out.size(), stdout);
  return 0;
}
