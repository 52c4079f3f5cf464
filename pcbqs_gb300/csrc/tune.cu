// The autotuner's memory (declared in tune.cuh) and its C ABI: entries "<device name>/<SM count>/<key>" -> choice,
// a text file of tab-separated lines when persistence is on.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>

#include "../../include/pcbqs_gb300.h"
#include "common.cuh"
#include "tune.cuh"

namespace pq {

namespace {

std::mutex g_mutex;
std::map<std::string, int> g_entries;
std::string g_path;
bool g_env_read = false;

// "<name>/<SM count>/" of the current device, looked up once per device (a lookup runs on every tuned call)
std::string device_prefix() {
    constexpr int MAX_DEVICES = 64;
    static std::mutex prefix_mutex;
    static std::string prefixes[MAX_DEVICES];
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) return "unknown/0/";
    std::lock_guard<std::mutex> lock(prefix_mutex);
    if (device >= 0 && device < MAX_DEVICES && !prefixes[device].empty()) return prefixes[device];
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return "unknown/0/";
    std::string name = prop.name;
    for (char &c : name)
        if (c == '\t' || c == '\n' || c == '/') c = ' ';
    name += "/" + std::to_string(prop.multiProcessorCount) + "/";
    if (device >= 0 && device < MAX_DEVICES) prefixes[device] = name;
    return name;
}

// Merges the file's entries (lines "key<TAB>value"); a missing file is an empty one. Caller holds g_mutex.
bool load_locked(const std::string &path) {
    FILE *f = std::fopen(path.c_str(), "r");
    if (!f) return true;
    char line[1024];
    bool ok = true;
    while (std::fgets(line, sizeof line, f)) {
        std::string s(line);
        while (!s.empty() && (s.back() == '\n' || s.back() == '\r')) s.pop_back();
        if (s.empty()) continue;
        const size_t tab = s.rfind('\t');
        if (tab == std::string::npos || tab == 0) {
            ok = false;
            continue;
        }
        char *end = nullptr;
        const long v = std::strtol(s.c_str() + tab + 1, &end, 10);
        if (!end || *end != '\0' || v < -1 || v > 1000000000L) {
            ok = false;
            continue;
        }
        g_entries[s.substr(0, tab)] = (int)v;
    }
    std::fclose(f);
    return ok;
}

// Writes every entry to a temporary file beside the tuning file, then renames it over (readers never see a half
// written file). Caller holds g_mutex.
bool save_locked() {
    if (g_path.empty()) return true;
    const std::string tmp = g_path + ".tmp";
    FILE *f = std::fopen(tmp.c_str(), "w");
    if (!f) return false;
    for (const auto &kv : g_entries) std::fprintf(f, "%s\t%d\n", kv.first.c_str(), kv.second);
    const bool ok = std::fclose(f) == 0;
    return ok && std::rename(tmp.c_str(), g_path.c_str()) == 0;
}

void read_env_locked() {
    if (g_env_read) return;
    g_env_read = true;
    const char *env = std::getenv("PCBQS_GB300_TUNE_FILE");
    if (env && *env && g_path.empty()) {
        g_path = env;
        load_locked(g_path);
    }
}

}  // namespace

int tune_get(const std::string &key) {
    const std::string full = device_prefix() + key;
    std::lock_guard<std::mutex> lock(g_mutex);
    read_env_locked();
    auto it = g_entries.find(full);
    return it == g_entries.end() ? -1 : it->second;
}

void tune_put(const std::string &key, int value) {
    const std::string full = device_prefix() + key;
    std::lock_guard<std::mutex> lock(g_mutex);
    read_env_locked();
    g_entries[full] = value;
    save_locked();
}

}  // namespace pq

extern "C" int pcbqs_gb300_tune_file(const char *path) {
    std::lock_guard<std::mutex> lock(pq::g_mutex);
    pq::g_env_read = true;                      // an explicit choice overrides the environment
    pq::g_path = path ? path : "";
    if (pq::g_path.empty()) return pq::OK;
    if (!pq::load_locked(pq::g_path)) return pq::fail(pq::ERR_ARGUMENT, "tune_file: malformed lines in %s", path);
    if (!pq::save_locked()) return pq::fail(pq::ERR_ARGUMENT, "tune_file: cannot write %s", path);
    return pq::OK;
}

extern "C" int pcbqs_gb300_tune_lookup(const char *key, int32_t *value) {
    if (!key || !value) return pq::fail(pq::ERR_ARGUMENT, "tune_lookup: null argument");
    const int v = pq::tune_get(key);
    *value = v;
    return v < 0 ? pq::fail(pq::ERR_ARGUMENT, "tune_lookup: no choice recorded for '%s'", key) : pq::OK;
}

extern "C" int pcbqs_gb300_tune_record(const char *key, int32_t value) {
    if (!key || !*key || value < 0 || std::strchr(key, '\t') || std::strchr(key, '\n'))
        return pq::fail(pq::ERR_ARGUMENT, "tune_record: a key without tabs or newlines and a value >= 0");
    pq::tune_put(key, value);
    return pq::OK;
}

extern "C" int64_t pcbqs_gb300_tune_count(void) {
    std::lock_guard<std::mutex> lock(pq::g_mutex);
    return (int64_t)pq::g_entries.size();
}

extern "C" void pcbqs_gb300_tune_clear(void) {
    std::lock_guard<std::mutex> lock(pq::g_mutex);
    pq::g_entries.clear();
}
