// A C++ caller of the drop-in boundary, written the way a program of the
// reference calls form_beams (cpu.cxx:48-67): sizes set once, std::vector
// storage (pageable host memory), then the reference's own checksum step
// (check(), arraysizes.cxx:79) on J.  Inputs are the seeded generator's bytes
// and the setup() gains.  Prints "status <n>" and exits 2 when a call fails;
// otherwise prints J's adler32 from form_beams + bf_adler32_host and from
// bf_form_beams_adler.
//
// usage: abi_caller ntimes nfrequencies ndishes npolarizations nbeams seed
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "beamform.h"

int main(int argc, char **argv) {
  if (argc != 7) {
    std::fprintf(stderr, "usage: %s T F D P B seed\n", argv[0]);
    return 1;
  }
  const bf_dims dims{std::atoll(argv[1]), std::atoll(argv[2]), std::atoll(argv[3]), std::atoll(argv[4]),
                     std::atoll(argv[5])};
  const uint64_t seed = std::strtoull(argv[6], nullptr, 10);
  std::vector<uint8_t> E(dims.ntimes * dims.nfrequencies * dims.ndishes * dims.npolarizations);
  std::vector<uint8_t> A(dims.nfrequencies * dims.nbeams * dims.ndishes);
  std::vector<float> G(dims.nfrequencies * dims.nbeams);
  std::vector<uint8_t> J(dims.nbeams * dims.nfrequencies * dims.npolarizations * dims.ntimes);
  if (bf_fill_random_host(E.data(), E.size(), seed, 0) != BF_OK || bf_fill_random_host(A.data(), A.size(), seed, 1) != BF_OK ||
      bf_gains_host(&dims, G.data()) != BF_OK || bf_set_dims(&dims) != BF_OK) {
    std::printf("status setup\n");
    return 2;
  }

  form_beams(J.data(), E.data(), A.data(), G.data());  // the reference's call
  if (bf_last_status() != BF_OK) {
    std::printf("status %d %s\n", bf_last_status(), bf_status_string(bf_last_status()));
    return 2;
  }
  uint32_t sum = 0;
  if (bf_adler32_host(J.data(), J.size(), &sum) != BF_OK) return 2;
  std::printf("adler32 0x%08x\n", sum);

  uint32_t fused = 0;
  const int st = bf_form_beams_adler(&dims, J.data(), E.data(), A.data(), G.data(), BF_A_LINEAR, BF_J_LINEAR,
                                     BF_PTR_HOST, &fused, nullptr);
  if (st != BF_OK) {
    std::printf("status %d %s\n", st, bf_status_string(st));
    return 2;
  }
  std::printf("fused 0x%08x\n", fused);
  return 0;
}
