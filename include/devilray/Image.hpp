// Image.hpp -- PNG output of RGBA8 pixels (the savePNG of the reference's
// include/Image.hpp), written without compression (stored deflate blocks).
#pragma once

#include "Utils.hpp"

#include <cstdint>
#include <string>
#include <vector>

void savePNG(const std::string &path, const std::vector<uint32_t> &pixels, Size2i size);
