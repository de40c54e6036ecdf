// Decodes a PNG with the library's reader and writes "width height channels
// bit_depth" on stdout and the samples (uint16, host order) to a file.
#include <cstdio>
#include <exception>
#include <fstream>
#include <iostream>

#include "png.h"

int main(int argc, char **argv) {
  if (argc < 3) return 2;
  try {
    kf::png::Image im = kf::png::read(argv[1]);
    std::cout << im.width << " " << im.height << " " << im.channels << " " << im.bit_depth << std::endl;
    std::ofstream o(argv[2], std::ios::binary);
    o.write((const char *)im.samples.data(), im.samples.size() * sizeof(uint16_t));
  } catch (const std::exception &e) {
    std::cerr << e.what() << std::endl;
    return 1;
  }
  return 0;
}
