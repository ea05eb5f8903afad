// Driver linked with the reference's LinearScan/gloveparser.cu (compiled from the
// read-only reference tree into oracle/_ref/) to dump what its text reader makes of a
// file, as golden vectors for the engine's reader.  Usage: parse_driver <file> > out.bin
// Output: int32 n, int32 d, then n * d float32 values.  Only files whose lines commit
// exactly n * d values are meaningful (the reader leaves other entries unset).
#include <cstdio>
#include <cstdlib>

float* parseFile(char* path, int& n, int& dimensions);

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  int n = 0, d = 0;
  float* v = parseFile(argv[1], n, d);
  fwrite(&n, sizeof n, 1, stdout);
  fwrite(&d, sizeof d, 1, stdout);
  fwrite(v, sizeof(float), (size_t)n * d, stdout);
  free(v);
  return 0;
}
