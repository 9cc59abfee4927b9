// Thread-local "last error" shared by every translation unit of libisti
// (the renderer, the image codecs and the dataset reader).
#pragma once

#include "isti.h"

#include <string>

namespace isti
{
// Stores `msg` as the calling thread's isti_last_error() and returns `s`.
isti_status set_error(isti_status s, const std::string &msg);

// Threads one image decode may use on the calling thread (0 = as many as useful, up
// to 8).  Callers that already decode several files at once set 1 on their workers.
void set_decode_threads(int n);
} // namespace isti
