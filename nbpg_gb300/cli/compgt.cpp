// nbpg_compgt: drop-in for the reference's CompGT (data_tools/ANNs/data_proc/CompGT.cpp:136-165),
// same flags (--base_path --query_path --gt_path --k --use_mips), same .gt output
// ([nq u32][k u32][ids u32][dists f32], CompGT.cpp:126-133), computed by nbpg_gt on the GPU
// in CompGT-compatible mode.  --exact keeps the true (dist, id) top-k instead.
#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

#include "../../include/nbpg.h"
#include "flags.h"

using namespace nbpg_cli;

static bool read_bin(const std::string &p, uint32_t &n, uint32_t &d, std::vector<uint8_t> &rows, size_t elem)
{
    std::ifstream f(p, std::ios::binary);
    if (!f) return false;
    f.read(reinterpret_cast<char *>(&n), 4);
    f.read(reinterpret_cast<char *>(&d), 4);
    rows.resize(size_t(n) * d * elem);
    f.read(reinterpret_cast<char *>(rows.data()), rows.size());
    return bool(f);
}

int main(int argc, char **argv)
{
    std::string base_path, query_path, gt_path;
    bool use_mips = false, exact = false;
    uint32_t k = 100;
    Flags fl;
    fl.opt("--base_path", base_path);
    fl.opt("--query_path", query_path);
    fl.opt("--gt_path", gt_path);
    fl.flag("--use_mips", use_mips);
    fl.opt("--k", k);
    fl.flag("--exact", exact);
    if (!fl.parse(argc, argv)) return 106;
    uint32_t dtype;
    if (ends_with(base_path, ".u8bin")) dtype = NBPG_U8;
    else if (ends_with(base_path, ".i8bin")) dtype = NBPG_I8;
    else if (ends_with(base_path, ".fbin") || ends_with(base_path, ".bin")) {
        std::fprintf(stderr, "nbpg_compgt: float vectors are not supported on the GPU path\n");
        return 2;
    } else return 0;  // the reference silently does nothing for other extensions
    uint32_t n, d, nq, dq;
    std::vector<uint8_t> base, q;
    if (!read_bin(base_path, n, d, base, 1) || !read_bin(query_path, nq, dq, q, 1) || d != dq) {
        std::fprintf(stderr, "nbpg_compgt: cannot read %s / %s\n", base_path.c_str(), query_path.c_str());
        return 1;
    }
    std::vector<uint32_t> ids(size_t(nq) * k);
    std::vector<float> dists(size_t(nq) * k);
    nbpg_status s = nbpg_gt(dtype, use_mips ? NBPG_IP : NBPG_L2, d, base.data(), n, q.data(), nq, k,
                            exact ? NBPG_GT_EXACT : NBPG_GT_COMPGT, ids.data(), dists.data(), 0);
    if (s != NBPG_OK) { std::fprintf(stderr, "nbpg_compgt: %s\n", nbpg_last_error()); return 1; }
    std::ofstream w(gt_path, std::ios::binary);
    w.write(reinterpret_cast<const char *>(&nq), 4);
    w.write(reinterpret_cast<const char *>(&k), 4);
    w.write(reinterpret_cast<const char *>(ids.data()), ids.size() * 4);
    w.write(reinterpret_cast<const char *>(dists.data()), dists.size() * 4);
    return w ? 0 : 1;
}
