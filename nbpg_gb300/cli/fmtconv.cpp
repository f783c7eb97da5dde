// nbpg_fmtconv: drop-in for the reference's FmtConv (data_tools/ANNs/data_proc/FmtConv.cpp:133-163):
// subcommands vec2bin (.fvecs -> .fbin), fbin2u8bin (truncate floats in [0, 256)) and
// u8bin2u4bin (keep the high nibble of each pair), each with --ifile --ofile, same outputs.
// The conversions run on the GPU (nbpg_f32_to_u8, nbpg_u8_to_u4); vec2bin is a file reshape.
#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

#include "../../include/nbpg.h"
#include "flags.h"

using namespace nbpg_cli;

static bool read_head(std::ifstream &r, uint32_t &n, uint32_t &d)
{
    r.read(reinterpret_cast<char *>(&n), 4);
    r.read(reinterpret_cast<char *>(&d), 4);
    return bool(r);
}

// FmtConv.cpp:18-61: rows of [dims u32][dims f32]; n = file length / (4 dims + 4)
static int vec2bin(const std::string &ifile, const std::string &ofile)
{
    std::ifstream r(ifile, std::ios::binary | std::ios::ate);
    if (!r) { std::fprintf(stderr, "nbpg_fmtconv: cannot read %s\n", ifile.c_str()); return 1; }
    const uint64_t len = uint64_t(r.tellg());
    r.seekg(0);
    uint32_t dims = 0;
    r.read(reinterpret_cast<char *>(&dims), 4);
    r.seekg(0);
    const uint32_t n = dims ? uint32_t(len / (4ull * dims + 4)) : 0;
    std::ofstream w(ofile, std::ios::binary);
    w.write(reinterpret_cast<const char *>(&n), 4);
    w.write(reinterpret_cast<const char *>(&dims), 4);
    std::vector<float> row(dims);
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t d = 0;
        r.read(reinterpret_cast<char *>(&d), 4);
        r.read(reinterpret_cast<char *>(row.data()), size_t(dims) * 4);
        w.write(reinterpret_cast<const char *>(row.data()), size_t(dims) * 4);
    }
    return w ? 0 : 1;
}

static int fbin2u8bin(const std::string &ifile, const std::string &ofile)
{
    std::ifstream r(ifile, std::ios::binary);
    uint32_t n, d;
    if (!r || !read_head(r, n, d)) { std::fprintf(stderr, "nbpg_fmtconv: cannot read %s\n", ifile.c_str()); return 1; }
    std::vector<float> in(size_t(n) * d);
    r.read(reinterpret_cast<char *>(in.data()), in.size() * 4);
    std::vector<uint8_t> out(in.size());
    if (nbpg_f32_to_u8(in.data(), n, d, out.data(), 0) != NBPG_OK) {
        std::fprintf(stderr, "nbpg_fmtconv: %s\n", nbpg_last_error());
        return 1;
    }
    std::ofstream w(ofile, std::ios::binary);
    w.write(reinterpret_cast<const char *>(&n), 4);
    w.write(reinterpret_cast<const char *>(&d), 4);
    w.write(reinterpret_cast<const char *>(out.data()), out.size());
    return w ? 0 : 1;
}

static int u8bin2u4bin(const std::string &ifile, const std::string &ofile)
{
    std::ifstream r(ifile, std::ios::binary);
    uint32_t n, d;
    if (!r || !read_head(r, n, d)) { std::fprintf(stderr, "nbpg_fmtconv: cannot read %s\n", ifile.c_str()); return 1; }
    std::vector<uint8_t> in(size_t(n) * d);
    r.read(reinterpret_cast<char *>(in.data()), in.size());
    const uint32_t half = d >> 1;
    std::vector<uint8_t> out(size_t(n) * half);
    if (n && d >= 2 && nbpg_u8_to_u4(in.data(), n, d, out.data(), 0) != NBPG_OK) {
        std::fprintf(stderr, "nbpg_fmtconv: %s\n", nbpg_last_error());
        return 1;
    }
    std::ofstream w(ofile, std::ios::binary);
    w.write(reinterpret_cast<const char *>(&n), 4);
    w.write(reinterpret_cast<const char *>(&half), 4);
    w.write(reinterpret_cast<const char *>(out.data()), out.size());
    return w ? 0 : 1;
}

int main(int argc, char **argv)
{
    if (argc < 2) { std::fprintf(stderr, "usage: nbpg_fmtconv {vec2bin|fbin2u8bin|u8bin2u4bin} --ifile X --ofile Y\n"); return 106; }
    const std::string cmd = argv[1];
    std::string ifile, ofile;
    Flags fl;
    fl.opt("--ifile", ifile);
    fl.opt("--ofile", ofile);
    if (!fl.parse(argc - 1, argv + 1)) return 106;
    if (cmd == "vec2bin") return vec2bin(ifile, ofile);
    if (cmd == "fbin2u8bin") return fbin2u8bin(ifile, ofile);
    if (cmd == "u8bin2u4bin") return u8bin2u4bin(ifile, ofile);
    std::fprintf(stderr, "nbpg_fmtconv: unknown subcommand %s\n", cmd.c_str());
    return 106;
}
