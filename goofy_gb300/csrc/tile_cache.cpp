// tile_cache.cpp -- the autotuner's results kept on disk, per GPU model.
//
// No reference counterpart: the reference's encoder has no launch shape to
// tune (goofy_tc.h runs one fixed SSE2 loop).  The fastest image-kernel tile
// differs between GB300 boxes (the register-loading BC1 grid took 39.5-51 us
// at 8192x8192 for the same shape), so goofy_gpu_autotune records its pick
// here, and goofy_gpu_init / the first call of a process (the drop-in
// included) install the recorded tiles instead of the compiled defaults.
//
// The file is plain text, one entry per line, '|'-separated:
//     v1|<GPU name>|<SM count>|<codec: bc1, etc1s, both>|<threads>|<blocks a thread>|<mode>|<us>
// '#' starts a comment line.  A line that does not parse, names a tile the
// kernels cannot run, or belongs to another GPU model is ignored.  Writers
// rewrite the whole file into a temporary sibling and rename it over the old
// one, so readers never see half a file.
#include "tile_cache.h"

#include <sys/stat.h>
#include <unistd.h>

#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <mutex>
#include <sstream>
#include <vector>

namespace goofy_gpu {

namespace {

constexpr const char* kVersion = "v1";
const char* const kCodecNames[3] = {"bc1", "etc1s", "both"};

std::mutex g_path_mu;
bool g_path_set = false;  // set_tile_cache_path was called
std::string g_path;

std::vector<std::string> split(const std::string& s, char sep)
{
    std::vector<std::string> out;
    size_t a = 0;
    for (;;) {
        const size_t b = s.find(sep, a);
        out.push_back(s.substr(a, b == std::string::npos ? std::string::npos : b - a));
        if (b == std::string::npos) return out;
        a = b + 1;
    }
}

bool parse_u32(const std::string& s, uint32_t* v)
{
    if (s.empty() || s.size() > 9) return false;
    uint32_t x = 0;
    for (char c : s) {
        if (c < '0' || c > '9') return false;
        x = x * 10 + (uint32_t)(c - '0');
    }
    *v = x;
    return true;
}

int codec_index(const std::string& s)
{
    for (int i = 0; i < 3; ++i)
        if (s == kCodecNames[i]) return i;
    return -1;
}

// A parsed entry, or false for a line to ignore.
struct Entry {
    std::string gpu;
    uint32_t sms = 0;
    int codec = -1;
    Tile tile{0, 0, 0};
};

bool parse_line(const std::string& line, Entry* e)
{
    if (line.empty() || line[0] == '#') return false;
    const std::vector<std::string> f = split(line, '|');
    if (f.size() != 8 || f[0] != kVersion || f[1].empty()) return false;
    e->gpu = f[1];
    e->codec = codec_index(f[3]);
    if (e->codec < 0) return false;
    if (!parse_u32(f[2], &e->sms) || !parse_u32(f[4], &e->tile.threads) || !parse_u32(f[5], &e->tile.bpt) ||
        !parse_u32(f[6], &e->tile.persistent))
        return false;
    if (!tile_valid(e->tile) || (e->codec == 2 && (e->tile.bpt > 2 || e->tile.persistent == 1))) return false;
    char* end = nullptr;
    const double us = std::strtod(f[7].c_str(), &end);
    return end && *end == '\0' && us > 0.0;
}

// '|' and line breaks cannot appear inside a field.
std::string clean(const std::string& s)
{
    std::string out = s;
    for (char& c : out)
        if (c == '|' || c == '\n' || c == '\r') c = '_';
    return out;
}

void make_parent_dirs(const std::string& path)
{
    for (size_t i = 1; i < path.size(); ++i)
        if (path[i] == '/') {
            const std::string dir = path.substr(0, i);
            if (mkdir(dir.c_str(), 0755) != 0 && errno != EEXIST) return;
        }
}

}  // namespace

std::string tile_cache_path()
{
    {
        std::lock_guard<std::mutex> lk(g_path_mu);
        if (g_path_set) return g_path;
    }
    if (const char* env = std::getenv("GOOFY_TILE_CACHE")) return env;  // "" disables the cache
    if (const char* xdg = std::getenv("XDG_CACHE_HOME"); xdg && *xdg)
        return std::string(xdg) + "/goofy_gb300/tiles.txt";
    if (const char* home = std::getenv("HOME"); home && *home) return std::string(home) + "/.cache/goofy_gb300/tiles.txt";
    return "";
}

void set_tile_cache_path(const char* path)
{
    std::lock_guard<std::mutex> lk(g_path_mu);
    g_path_set = path != nullptr;
    g_path = path ? path : "";
}

bool tile_cache_lookup(const std::string& path, const std::string& gpu, uint32_t sms, int codec, Tile* out)
{
    if (path.empty() || codec < 0 || codec > 2) return false;
    std::ifstream f(path);
    if (!f) return false;
    const std::string name = clean(gpu);
    bool found = false;
    std::string line;
    Entry e;
    while (std::getline(f, line)) {  // the last valid entry for this GPU and codec wins
        if (parse_line(line, &e) && e.gpu == name && e.sms == sms && e.codec == codec) {
            *out = e.tile;
            found = true;
        }
    }
    return found;
}

int tile_cache_store(const std::string& path, const std::string& gpu, uint32_t sms, int codec, const Tile& t,
                     float us)
{
    if (path.empty()) return fail(GOOFY_ERR_INVALID, "tile cache: no path (disabled)");
    if (gpu.empty() || codec < 0 || codec > 2 || !tile_valid(t) || !(us > 0.f))
        return fail(GOOFY_ERR_INVALID, "tile cache: bad entry");
    const std::string name = clean(gpu);
    std::vector<std::string> keep;
    {
        std::ifstream f(path);
        std::string line;
        Entry e;
        while (f && std::getline(f, line)) {
            if (!line.empty() && line[0] == '#') continue;  // the header is rewritten below
            if (parse_line(line, &e) && e.gpu == name && e.sms == sms && e.codec == codec) continue;  // replaced
            if (!line.empty()) keep.push_back(line);
        }
    }
    std::ostringstream body;
    body << "# goofy_gb300 tuned image-kernel tiles: " << kVersion
         << "|gpu|sms|codec|threads|blocks a thread|mode|us\n";
    for (const std::string& l : keep) body << l << "\n";
    char usbuf[32];
    std::snprintf(usbuf, sizeof usbuf, "%.3f", (double)us);
    body << kVersion << "|" << name << "|" << sms << "|" << kCodecNames[codec] << "|" << t.threads << "|" << t.bpt << "|"
         << t.persistent << "|" << usbuf << "\n";
    make_parent_dirs(path);
    const std::string tmp = path + ".tmp." + std::to_string((long)getpid());
    {
        std::ofstream o(tmp, std::ios::trunc);
        if (!o || !(o << body.str()) || !o.flush()) {
            std::remove(tmp.c_str());
            return fail(GOOFY_ERR_INVALID, "tile cache: cannot write the file");
        }
    }
    if (std::rename(tmp.c_str(), path.c_str()) != 0) {
        std::remove(tmp.c_str());
        return fail(GOOFY_ERR_INVALID, "tile cache: cannot replace the file");
    }
    return GOOFY_OK;
}

}  // namespace goofy_gpu
