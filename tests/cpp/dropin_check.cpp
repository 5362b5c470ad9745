// A caller of the drop-in C++ classes (include/ctsim_gpu.h), built and run by
// tests/test_gpu_dropin_cpp.py:
//   dropin_check polar PJFILE NX NY INTERP OUT.f32   Projections::convertPolar
//   dropin_check comp A.if B.if                      ImageFile::printComparativeStatistics
//   dropin_check sub A.if B.if OUT.if                ImageFile::subtractImages + labelsCopy
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>

#include "ctsim_gpu.h"

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  if (!std::strcmp(argv[1], "polar") && argc == 7) {
    Projections pj;
    if (!pj.read(argv[2])) return 3;
    ImageFile im(std::atoi(argv[3]), std::atoi(argv[4]));
    if (!pj.convertPolar(im, Projections::convertInterpNameToID(argv[5]))) return 4;
    FILE* f = std::fopen(argv[6], "wb");
    if (!f) return 5;
    std::fwrite(im.data(), sizeof(float), (size_t)im.nx() * im.ny(), f);
    std::fclose(f);
    return 0;
  }
  if (!std::strcmp(argv[1], "comp") && argc == 4) {
    ImageFile a, b;
    if (!a.fileRead(argv[2]) || !b.fileRead(argv[3])) return 3;
    return a.printComparativeStatistics(b, std::cout) ? 0 : 4;
  }
  if (!std::strcmp(argv[1], "sub") && argc == 5) {
    ImageFile a, b;
    if (!a.fileRead(argv[2]) || !b.fileRead(argv[3])) return 3;
    ImageFile out(a.nx(), a.ny());
    if (!a.subtractImages(b, out)) return 4;
    out.labelsCopy(a, "if2 file 1: ");
    out.labelsCopy(b, "if2 file 2: ");
    return out.fileWrite(argv[4]) ? 0 : 5;
  }
  return 2;
}
