// ref_io_main.cxx -- TEST INFRASTRUCTURE ONLY.
//
// Driver that links against the reference's own form_beams (cpu.cxx:15-46),
// compiled unmodified from the reference sources by oracle/build_ref.sh with a
// generated arraysizes.hxx that fixes the shape.  It reads E, A and G from
// files, calls the reference function once, and writes J, so the oracle's
// restatement can be compared with the reference byte for byte on seeded
// inputs.  Built only where the reference sources are present.
#include <cstdio>
#include <cstdlib>
#include <vector>

// Declared with the reference's own signature (cpu.cxx:15-16); the types and
// the size constants come from the reference headers on the include path.
void form_beams(ucomplex4 *restrict const Jarray, const ucomplex4 *restrict const Earray,
                const ucomplex4 *restrict const Aarray, const float *restrict Garray);

static bool read_file(const char *path, void *dst, size_t n) {
  FILE *fp = std::fopen(path, "rb");
  if (!fp) return false;
  const size_t got = std::fread(dst, 1, n, fp);
  std::fclose(fp);
  return got == n;
}

int main(int argc, char **argv) {
  if (argc != 5) {
    std::fprintf(stderr, "usage: %s E.bin A.bin G.bin J.out\n", argv[0]);
    return 2;
  }
  std::vector<ucomplex4> E(Esize / 2), A(Asize / 2), J(Jsize / 2);
  std::vector<float> G(Gsize);
  if (!read_file(argv[1], E.data(), E.size()) || !read_file(argv[2], A.data(), A.size()) ||
      !read_file(argv[3], G.data(), G.size() * sizeof(float))) {
    std::fprintf(stderr, "short input file\n");
    return 3;
  }
  const double t0 = gettime();
  form_beams(J.data(), E.data(), A.data(), G.data());
  const double t1 = gettime();
  FILE *fp = std::fopen(argv[4], "wb");
  if (!fp || std::fwrite(J.data(), 1, J.size(), fp) != J.size()) return 4;
  std::fclose(fp);
  std::printf("%.6f\n", t1 - t0);
  return 0;
}
