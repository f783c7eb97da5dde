// nbpg_pcacompress: drop-in for the reference's PCACompress (data_tools/ANNs/data_proc/
// PCACompress.cpp:85-108): same flags (--ifile --ofile --matFile --index_type), same
// input kinds (.fbin/.bin floats, .u8bin/.i8bin codes), same output chosen by the output
// extension (.u4bin/.i4bin: two 4-bit codes per byte; .u8bin/.i8bin: one code per byte;
// anything else: float values), same header ([n][dims] as uint32, or uint64 with
// --index_type uint64).  The projection and quantisation run on the GPU (nbpg_pca_encode).
#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

#include "../../include/nbpg.h"
#include "flags.h"

using namespace nbpg_cli;

// .mat (matrix.h:59-84): [d_out u32][d_in u32][has_bias bool][d_out x d_in f32][bias f32 x d_out]
static bool read_mat(const std::string &p, uint32_t &d_out, uint32_t &d_in, std::vector<float> &mat,
                     std::vector<float> &bias)
{
    std::ifstream f(p, std::ios::binary);
    if (!f) return false;
    uint8_t has_bias = 0;
    f.read(reinterpret_cast<char *>(&d_out), 4);
    f.read(reinterpret_cast<char *>(&d_in), 4);
    f.read(reinterpret_cast<char *>(&has_bias), 1);
    mat.resize(size_t(d_out) * d_in);
    f.read(reinterpret_cast<char *>(mat.data()), mat.size() * 4);
    bias.assign(d_out, 0.0f);
    if (has_bias) f.read(reinterpret_cast<char *>(bias.data()), size_t(d_out) * 4);
    return bool(f);
}

template <class I>
static int run(const std::string &ifile, const std::string &ofile, uint32_t d_out, uint32_t d_in,
               const std::vector<float> &mat, const std::vector<float> &bias)
{
    uint32_t in_dtype;
    size_t in_b = 1;
    if (ends_with(ifile, ".fbin") || ends_with(ifile, ".bin")) { in_dtype = NBPG_F32; in_b = 4; }
    else if (ends_with(ifile, ".u8bin")) in_dtype = NBPG_U8;
    else if (ends_with(ifile, ".i8bin")) in_dtype = NBPG_I8;
    else { std::fprintf(stderr, "nbpg_pcacompress: unsupported input %s\n", ifile.c_str()); return 1; }
    uint32_t out_dtype = NBPG_F32, chunk = 1;
    if (ends_with(ofile, ".u4bin")) { out_dtype = NBPG_U4; chunk = 2; }
    else if (ends_with(ofile, ".i4bin")) { out_dtype = NBPG_I4; chunk = 2; }
    else if (ends_with(ofile, ".u8bin")) out_dtype = NBPG_U8;
    else if (ends_with(ofile, ".i8bin")) out_dtype = NBPG_I8;
    std::ifstream r(ifile, std::ios::binary);
    if (!r) { std::fprintf(stderr, "nbpg_pcacompress: cannot read %s\n", ifile.c_str()); return 1; }
    I n = 0, dims = 0;
    r.read(reinterpret_cast<char *>(&n), sizeof(I));
    r.read(reinterpret_cast<char *>(&dims), sizeof(I));
    if (uint64_t(dims) != d_in) { std::fprintf(stderr, "nbpg_pcacompress: matrix expects %u dims, file has %llu\n", d_in,
                                                (unsigned long long)dims); return 1; }
    const I out_dims = I(d_out / chunk);
    std::ofstream w(ofile, std::ios::binary);
    w.write(reinterpret_cast<const char *>(&n), sizeof(I));
    w.write(reinterpret_cast<const char *>(&out_dims), sizeof(I));
    const size_t out_row = out_dtype == NBPG_F32 ? size_t(d_out) * 4 : size_t(out_dims);
    const uint64_t BLOCK = 1000000;
    std::vector<uint8_t> in, out;
    for (uint64_t p = 0; p < uint64_t(n); p += BLOCK) {
        const uint64_t cnt = std::min<uint64_t>(BLOCK, uint64_t(n) - p);
        in.resize(cnt * d_in * in_b);
        out.resize(cnt * out_row);
        r.read(reinterpret_cast<char *>(in.data()), in.size());
        if (!r) { std::fprintf(stderr, "nbpg_pcacompress: %s is truncated\n", ifile.c_str()); return 1; }
        const nbpg_status s = nbpg_pca_encode(in_dtype, in.data(), cnt, d_in, mat.data(), bias.data(), d_out,
                                              out_dtype, out.data(), 0);
        if (s != NBPG_OK) { std::fprintf(stderr, "nbpg_pcacompress: %s\n", nbpg_last_error()); return 1; }
        w.write(reinterpret_cast<const char *>(out.data()), out.size());
    }
    return w ? 0 : 1;
}

int main(int argc, char **argv)
{
    std::string ifile, ofile, mat_file, index_type = "uint32";
    Flags fl;
    fl.opt("--ifile", ifile);
    fl.opt("--ofile", ofile);
    fl.opt("--matFile", mat_file);
    fl.opt("--index_type", index_type);
    if (!fl.parse(argc, argv)) return 106;
    uint32_t d_out, d_in;
    std::vector<float> mat, bias;
    if (!read_mat(mat_file, d_out, d_in, mat, bias)) {
        std::fprintf(stderr, "nbpg_pcacompress: cannot read %s\n", mat_file.c_str());
        return 1;
    }
    if (index_type == "uint64") return run<uint64_t>(ifile, ofile, d_out, d_in, mat, bias);
    if (index_type == "uint32") return run<uint32_t>(ifile, ofile, d_out, d_in, mat, bias);
    return 0;  // the reference does nothing for other index types
}
