// Emits the reference test's known-answer inputs: integers 0..9 from one
// std::mt19937 seeded with 42 through std::uniform_int_distribution<int>(0, 9),
// drawn for A, then B, then C (tests/test-multiply.cpp:58-66, 269-271).
// Usage: kat_inputs <n_a> <n_b> <n_c>   -> n_a + n_b + n_c bytes on stdout.
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

int main(int argc, char** argv) {
  if (argc != 4) return 2;
  std::mt19937 rng(42);
  std::uniform_int_distribution<int> dist(0, 9);
  for (int i = 1; i <= 3; ++i) {
    long n = std::atol(argv[i]);
    std::vector<unsigned char> buf((size_t)n);
    for (long j = 0; j < n; ++j) buf[(size_t)j] = (unsigned char)dist(rng);
    fwrite(buf.data(), 1, buf.size(), stdout);
  }
  return 0;
}
