// Autotuning cache shared by the librsx handles (rsx_autotune.cpp).
#pragma once
#include <cuda_runtime.h>
#include <string>

namespace rsx {

std::string autotune_key(int device, const char *kind, long long size, int n_q, int n_types,
                         bool uniform, bool water);
bool autotune_lookup(const std::string &key, int *value);
void autotune_store(const std::string &key, int value);
void autotune_clear();

} // namespace rsx
