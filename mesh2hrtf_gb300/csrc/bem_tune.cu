// bem_tune.cu - the launch-shape tuner's cache.
//
// The library tunes launch shapes that leave every result bit unchanged: the
// persistent grids of the assembly (k_far and k_near resident blocks per SM)
// and the strip height of the complex64 matrix-vector product (rows per work
// item, which sets how finely a system's product spreads over the SMs).  The
// first assembly and the first solve of a key time every candidate with CUDA
// events and keep the fastest (bem_api.cu); this file holds the choices.
//
// Key: device model and SM count, size bucket (n rounded to a quarter power
// of two), precision and right-hand sides.  Choices live in memory and are
// appended to a text cache file, one line per choice, read at the first
// lookup: $BEM_GB300_TUNE_CACHE, else $XDG_CACHE_HOME/mesh2hrtf_gb300/tune.txt,
// else $HOME/.cache/mesh2hrtf_gb300/tune.txt.  BEM_GB300_TUNE=0 turns tuning
// off (the defaults run).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <sys/stat.h>
#include <tuple>

#include "../../include/bem_gb300.h"
#include "bem_internal.h"

namespace bem {
namespace {

using Key = std::tuple<std::string, int, int, int, int>;   // device, sms, bucket, prec, rhs

std::mutex g_mu;
std::map<Key, TuneChoice> g_cache;
bool g_loaded = false;

std::string device_tag(int *sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceProp p;
    std::string name = "unknown";
    *sms = 0;
    if (cudaGetDeviceProperties(&p, dev) == cudaSuccess) {
        name = p.name;
        *sms = p.multiProcessorCount;
    } else {
        cudaGetLastError();
    }
    for (char &c : name)
        if (c == ' ' || c == '\t') c = '_';
    return name;
}

std::string cache_path() {
    if (const char *p = std::getenv("BEM_GB300_TUNE_CACHE")) return p;
    std::string base;
    if (const char *x = std::getenv("XDG_CACHE_HOME")) base = x;
    else if (const char *h = std::getenv("HOME")) base = std::string(h) + "/.cache";
    else return std::string();
    return base + "/mesh2hrtf_gb300/tune.txt";
}

void make_dirs(const std::string &file) {
    for (size_t i = 1; i < file.size(); ++i)
        if (file[i] == '/') mkdir(file.substr(0, i).c_str(), 0755);
}

// line: v1 <device> <sms> <bucket> <prec> <rhs> asm <far> <near> <ms>
//   or: v1 <device> <sms> <bucket> <prec> <rhs> mv <strip> <ms>
void load_locked() {
    if (g_loaded) return;
    g_loaded = true;
    const std::string path = cache_path();
    if (path.empty()) return;
    FILE *f = std::fopen(path.c_str(), "r");
    if (!f) return;
    char dev[256], what[8];
    int sms, bucket, prec, rhs;
    char line[512];
    while (std::fgets(line, sizeof(line), f)) {
        if (std::sscanf(line, "v1 %255s %d %d %d %d %7s", dev, &sms, &bucket, &prec, &rhs, what) != 6) continue;
        TuneChoice &c = g_cache[Key(dev, sms, bucket, prec, rhs)];
        const char *rest = std::strstr(line, what) + std::strlen(what);
        if (!std::strcmp(what, "asm")) {
            int fa, ne;
            double ms;
            if (std::sscanf(rest, "%d %d %lf", &fa, &ne, &ms) == 3 && fa >= 1 && fa <= kFarPerSmMax && ne >= 1 &&
                ne <= 2) {
                c.asm_shape.far_per_sm = fa;
                c.asm_shape.near_per_sm = ne;
                c.asm_ms = ms;
                c.asm_tuned = true;
            }
        } else if (!std::strcmp(what, "mv")) {
            int strip;
            double ms;
            if (std::sscanf(rest, "%d %lf", &strip, &ms) == 2 && strip >= kTmaRows && strip <= kTmaStripMax &&
                strip % kTmaRows == 0) {
                c.mv_strip = strip;
                c.mv_ms = ms;
                c.mv_tuned = true;
            }
        }
    }
    std::fclose(f);
}

void append_line(const std::string &text) {
    const std::string path = cache_path();
    if (path.empty()) return;
    make_dirs(path);
    FILE *f = std::fopen(path.c_str(), "a");
    if (!f) return;
    std::fputs(text.c_str(), f);   // one short line per append
    std::fclose(f);
}

Key key_of(int n, int prec, int n_rhs) {
    int sms = 0;
    const std::string dev = device_tag(&sms);
    return Key(dev, sms, tune_bucket(n), prec, n_rhs < 1 ? 1 : n_rhs);
}

}  // namespace

bool tune_enabled() {
    const char *v = std::getenv("BEM_GB300_TUNE");
    return !(v && v[0] == '0');
}

int tune_bucket(int n) { return n <= 1 ? 0 : (int)std::lround(4.0 * std::log2((double)n)); }

TuneChoice tune_lookup(int n, int prec, int n_rhs) {
    if (!tune_enabled()) return TuneChoice();
    const Key k = key_of(n, prec, n_rhs);
    std::lock_guard<std::mutex> lk(g_mu);
    load_locked();
    auto it = g_cache.find(k);
    return it == g_cache.end() ? TuneChoice() : it->second;
}

void tune_store_asm(int n, int prec, int n_rhs, AsmShape s, double ms) {
    const Key k = key_of(n, prec, n_rhs);
    std::lock_guard<std::mutex> lk(g_mu);
    load_locked();
    TuneChoice &c = g_cache[k];
    c.asm_shape = s;
    c.asm_ms = ms;
    c.asm_tuned = true;
    char buf[512];
    std::snprintf(buf, sizeof(buf), "v1 %s %d %d %d %d asm %d %d %.6f\n", std::get<0>(k).c_str(), std::get<1>(k),
                  std::get<2>(k), prec, std::get<4>(k), s.far_per_sm, s.near_per_sm, ms);
    append_line(buf);
}

void tune_store_mv(int n, int prec, int n_rhs, int strip, double ms) {
    const Key k = key_of(n, prec, n_rhs);
    std::lock_guard<std::mutex> lk(g_mu);
    load_locked();
    TuneChoice &c = g_cache[k];
    c.mv_strip = strip;
    c.mv_ms = ms;
    c.mv_tuned = true;
    char buf[512];
    std::snprintf(buf, sizeof(buf), "v1 %s %d %d %d %d mv %d %.6f\n", std::get<0>(k).c_str(), std::get<1>(k),
                  std::get<2>(k), prec, std::get<4>(k), strip, ms);
    append_line(buf);
}

}  // namespace bem

extern "C" bem_status bem_tune_info(int32_t n_elem, int32_t precision, int32_t n_rhs, char *buf, int32_t len) {
    if (!buf || len <= 0) {
        bem::set_error("bem_tune_info: null buffer");
        return BEM_ERR_INVALID;
    }
    const bem::TuneChoice c = bem::tune_lookup(n_elem, precision, n_rhs);
    const bem::TuneChoice d;
    std::snprintf(buf, (size_t)len,
                  "{\"bucket\": %d, \"enabled\": %s, \"assembly\": {\"far_blocks_per_sm\": %d, "
                  "\"near_blocks_per_sm\": %d, \"tuned\": %s, \"ms\": %.6f}, \"product\": {\"strip_rows\": %d, "
                  "\"tuned\": %s, \"ms\": %.6f}, \"defaults\": {\"far_blocks_per_sm\": %d, \"near_blocks_per_sm\": %d, "
                  "\"strip_rows\": %d}}",
                  bem::tune_bucket(n_elem), bem::tune_enabled() ? "true" : "false", c.asm_shape.far_per_sm,
                  c.asm_shape.near_per_sm, c.asm_tuned ? "true" : "false", c.asm_ms, c.mv_strip,
                  c.mv_tuned ? "true" : "false", c.mv_ms, d.asm_shape.far_per_sm, d.asm_shape.near_per_sm,
                  d.mv_strip);
    return BEM_OK;
}
