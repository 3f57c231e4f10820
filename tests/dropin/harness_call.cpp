// harness_call.cpp -- TEST ONLY.  A C++ caller written the way the reference
// harness calls the encoder (Src/main.cpp:644 CompressFunc_t, :925-929), built
// against include/goofy_tc_gpu.h and linked with libgoofy_gb300.so instead of
// compiling GoofyTC/goofy_tc.h.
//
//   harness_call codes                         -> prints the return codes of bad sizes (no GPU needed)
//   harness_call encode IN W H STRIDE OUT_ETC OUT_DXT
//                                               -> encodes the raw RGBA8 rows in IN with both entry points
#include <cstdio>
#include <cstdlib>
#include <string_view>
#include <vector>

#include "goofy_tc_gpu.h"

typedef int (*CompressFunc_t)(unsigned char* result, const unsigned char* input, unsigned int width,
                              unsigned int height, unsigned int stride);

static bool read_file(const char* path, std::vector<unsigned char>& data)
{
    FILE* f = std::fopen(path, "rb");
    if (!f) return false;
    unsigned char buf[65536];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof buf, f)) > 0) data.insert(data.end(), buf, buf + n);
    std::fclose(f);
    return true;
}

static bool write_file(const char* path, const std::vector<unsigned char>& data)
{
    FILE* f = std::fopen(path, "wb");
    if (!f) return false;
    const bool ok = std::fwrite(data.data(), 1, data.size(), f) == data.size();
    return std::fclose(f) == 0 && ok;
}

int main(int argc, char** argv)
{
    const CompressFunc_t funcs[2] = {goofy::compressETC1, goofy::compressDXT1};
    if (argc == 2 && std::string_view(argv[1]) == "codes") {
        std::vector<unsigned char> in(64 * 64 * 4), out(64 * 64 / 2);
        for (CompressFunc_t f : funcs)
            std::printf("%d %d %d\n", f(out.data(), in.data(), 60, 64, 256), f(out.data(), in.data(), 64, 62, 256),
                        f(out.data(), in.data(), 8, 64, 256));
        return 0;
    }
    if (argc == 8 && std::string_view(argv[1]) == "encode") {
        std::vector<unsigned char> in;
        if (!read_file(argv[2], in)) return 2;
        const unsigned w = (unsigned)std::atoi(argv[3]), h = (unsigned)std::atoi(argv[4]),
                       stride = (unsigned)std::atoi(argv[5]);
        for (int k = 0; k < 2; ++k) {
            std::vector<unsigned char> out((size_t)(w / 4) * (h / 4) * 8);
            const int rc = funcs[k](out.data(), in.data(), w, h, stride);
            if (rc != 0) {
                std::printf("rc %d\n", rc);
                return 3;
            }
            if (!write_file(argv[6 + k], out)) return 4;
        }
        std::printf("ok\n");
        return 0;
    }
    return 1;
}
