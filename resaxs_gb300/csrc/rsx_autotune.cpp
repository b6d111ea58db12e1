// Autotuning cache for librsx: the winning tile shape of a problem class
// (the q-slab plan, and for the wide forward the pairs a thread steps
// together), chosen by timing the candidates on the device on first use.
// Stored as q_slab + 1000 * (pairs_per_step == 4).
//
// Key: device name | kind | log2 size bucket | n_q | n_types | uniform | water.
// The cache lives in the process; when RSX_AUTOTUNE_CACHE names a file it is
// also loaded from and appended to it (one "key value" line per entry).
#include "rsx_autotune.h"
#include "rsx.h"

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>

namespace rsx {

static bool valid_q_slab(long v)
{
    return v == 8 || v == 16 || v == 32 || v == 64 || v == 128 || v == 192 || v == 1128 ||
           v == 1192;
}

static std::mutex g_mu;
static std::map<std::string, int> g_cache;
static bool g_loaded = false;

static void load_file_locked()
{
    if (g_loaded)
        return;
    g_loaded = true;
    const char *path = std::getenv("RSX_AUTOTUNE_CACHE");
    if (!path || !*path)
        return;
    std::ifstream in(path);
    std::string line;
    while (std::getline(in, line)) {
        const auto sp = line.rfind(' ');
        if (sp == std::string::npos)
            continue;
        // the file is outside the library's control: keep only tile shapes
        // that librsx has kernels for, so an edited or damaged line can
        // never select a kernel shape that does not exist
        char *end = nullptr;
        const long v = std::strtol(line.c_str() + sp + 1, &end, 10);
        if (end == line.c_str() + sp + 1 || *end != '\0' || !valid_q_slab(v))
            continue;
        g_cache[line.substr(0, sp)] = (int)v;
    }
}

std::string autotune_key(int device, const char *kind, long long size, int n_q, int n_types,
                         bool uniform, bool water)
{
    cudaDeviceProp prop;
    std::string name = "dev";
    if (cudaGetDeviceProperties(&prop, device) == cudaSuccess)
        name = prop.name;
    for (auto &c : name)
        if (c == ' ')
            c = '_';
    int bucket = 0;
    while ((1LL << (bucket + 1)) <= size)
        ++bucket;
    std::ostringstream k;
    k << name << '|' << kind << '|' << bucket << '|' << n_q << '|' << n_types << '|' << uniform
      << '|' << water;
    return k.str();
}

bool autotune_lookup(const std::string &key, int *value)
{
    std::lock_guard<std::mutex> lk(g_mu);
    load_file_locked();
    auto it = g_cache.find(key);
    if (it == g_cache.end())
        return false;
    *value = it->second;
    return true;
}

void autotune_store(const std::string &key, int value)
{
    std::lock_guard<std::mutex> lk(g_mu);
    load_file_locked();
    g_cache[key] = value;
    const char *path = std::getenv("RSX_AUTOTUNE_CACHE");
    if (path && *path) {
        std::ofstream out(path, std::ios::app);
        out << key << ' ' << value << '\n';
    }
}

void autotune_clear()
{
    std::lock_guard<std::mutex> lk(g_mu);
    g_cache.clear();
    g_loaded = true; // do not reload the file after an explicit clear
}

} // namespace rsx

extern "C" void rsx_autotune_clear(void) { rsx::autotune_clear(); }

extern "C" int rsx_debug_autotune_lookup(const char *key, int *q_slab)
{
    int v = 0;
    if (!key || !q_slab || !rsx::autotune_lookup(key, &v))
        return 0;
    *q_slab = v;
    return 1;
}
