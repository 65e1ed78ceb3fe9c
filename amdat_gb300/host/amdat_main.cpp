// amdat_gb300 command-line driver: runs an AMDAT input script's hot-path
// commands on one GPU (src/amdat.cpp:30-142 flags -i <file>; -d <device>).
#include <cstdlib>
#include <cstring>
#include <iostream>

#include "../../include/amdat_gb300.h"

int main(int argc, char** argv) {
  const char* input = nullptr;
  int device = 0;
  for (int i = 1; i < argc; ++i) {
    if (!std::strcmp(argv[i], "-i") && i + 1 < argc) input = argv[++i];
    else if (!std::strcmp(argv[i], "-d") && i + 1 < argc) device = std::atoi(argv[++i]);
    else if (!std::strcmp(argv[i], "-v")) {
      std::cout << amdat_version() << "\n";
      return 0;
    } else if (!std::strcmp(argv[i], "-n") && i + 1 < argc) {
      ++i;  // thread count: the GPU engine ignores it
    }
  }
  if (!input) {
    std::cerr << "usage: amdat_gb300 -i <input script> [-d <device>]\n";
    return 2;
  }
  const amdat_status s = amdat_run_script(input, device);
  if (s != AMDAT_OK) {
    std::cerr << "Error: " << amdat_script_error() << "\n";
    return 1;
  }
  std::cout << "Program completed successfully.\n";
  return 0;
}
