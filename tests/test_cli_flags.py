"""The drop-in executables accept every flag that the reference's drivers declare, in the
same syntax (--name value, --name=value, bare boolean flags), and reject an unknown one
with CLI11's exit code for an unexpected argument (106).  Runs on the CPU: given no input
of a known extension, each drop-in returns right after parsing, as the reference does.
Where the reference sources are present, the lists below are checked against the
uncommented add_option / add_flag declarations of each driver."""
import os
import re
import subprocess

import pytest

# (reference driver, options taking a value, boolean flags)
DRIVERS = {
    # data_tools/ANNs/Vamana.cpp:59-124
    "nbpg_vamana": ("data_tools/ANNs/Vamana.cpp",
                    ["--quant_base_path", "--pre_index_path", "--index_path", "--R", "--L", "--limit", "--VL",
                     "--top_degree", "--num_passes", "--num_split", "--dir_bias_scale", "--max_alpha", "--min_alpha",
                     "--max_cos_angle", "--min_cos_angle", "--base_path", "--query_path", "--quant_query_path",
                     "--gt_path", "--res_path", "--k", "--Q", "--rerank_factor", "--q_num"],
                    ["--dynamic_prune", "--use_mips", "--rebuild", "--rand_sp", "--cache_raw", "--verbose"]),
    # data_tools/ANNs/FGIM/FGIM.cpp:67-132 (no cos-angle bounds)
    "nbpg_fgim": ("data_tools/ANNs/FGIM/FGIM.cpp",
                  ["--quant_base_path", "--pre_index_path", "--index_path", "--R", "--L", "--limit", "--VL",
                   "--top_degree", "--num_passes", "--num_split", "--dir_bias_scale", "--max_alpha", "--min_alpha",
                   "--base_path", "--query_path", "--quant_query_path", "--gt_path", "--res_path", "--k", "--Q",
                   "--rerank_factor", "--q_num"],
                  ["--dynamic_prune", "--use_mips", "--rebuild", "--rand_sp", "--cache_raw", "--verbose"]),
    # data_tools/ANNs/HNSW/HNSW.cpp:53-125
    "nbpg_hnsw": ("data_tools/ANNs/HNSW/HNSW.cpp",
                  ["--quant_base_path", "--index_path", "--R", "--PR", "--L", "--limit", "--VL", "--alpha",
                   "--cos_angle", "--m_l", "--max_node_num", "--top_degree", "--hier_beamSize", "--base_path",
                   "--query_path", "--quant_query_path", "--gt_path", "--res_path", "--k", "--Q", "--rerank_factor",
                   "--q_num"],
                  ["--use_mips", "--rebuild", "--cache_raw", "--verbose"]),
    # data_tools/ANNs/data_proc/CompGT.cpp:141-148 (--data_type, --dist_func, --index_type are
    # commented out there, so the reference rejects them too)
    "nbpg_compgt": ("data_tools/ANNs/data_proc/CompGT.cpp", ["--base_path", "--query_path", "--gt_path", "--k"],
                    ["--use_mips"]),
    # data_tools/ANNs/data_proc/PCACompress.cpp:86-89
    "nbpg_pcacompress": ("data_tools/ANNs/data_proc/PCACompress.cpp", ["--ifile", "--ofile", "--matFile",
                                                                        "--index_type"], []),
}
# data_tools/ANNs/data_proc/FmtConv.cpp:141-151: three subcommands, each with --ifile and --ofile
FMTCONV = ("data_tools/ANNs/data_proc/FmtConv.cpp", ["vec2bin", "fbin2u8bin", "u8bin2u4bin"], ["--ifile", "--ofile"])


@pytest.fixture(scope="module")
def bindir():
    from nbpg_gb300 import build_ext
    exe = os.path.join(build_ext.OUT, "nbpg_vamana")
    if not os.path.exists(exe):
        build_ext.build()
    return build_ext.OUT


def _run(bindir, exe, args, cwd):
    return subprocess.run([os.path.join(bindir, exe), *args], capture_output=True, text=True, timeout=60, cwd=cwd)


@pytest.mark.parametrize("exe", sorted(DRIVERS))
def test_drop_in_accepts_every_reference_flag(bindir, tmp_path, exe):
    _, opts, flags = DRIVERS[exe]
    for o in opts:
        for args in ([o, "1"], [o + "=1"]):
            r = _run(bindir, exe, args, tmp_path)
            assert r.returncode != 106 and "not expected" not in r.stderr, (exe, args, r.stderr)
    for fl in flags:
        r = _run(bindir, exe, [fl], tmp_path)
        assert r.returncode != 106 and "not expected" not in r.stderr, (exe, fl, r.stderr)
    r = _run(bindir, exe, ["--no_such_flag", "1"], tmp_path)
    assert r.returncode == 106 and "--no_such_flag" in r.stderr


def test_fmtconv_subcommands(bindir, tmp_path):
    _, subs, opts = FMTCONV
    for sub in subs:
        for o in opts:
            r = _run(bindir, "nbpg_fmtconv", [sub, o, "1"], tmp_path)
            assert r.returncode != 106 and "not expected" not in r.stderr, (sub, o, r.stderr)
        assert _run(bindir, "nbpg_fmtconv", [sub, "--no_such_flag", "1"], tmp_path).returncode == 106
    assert _run(bindir, "nbpg_fmtconv", ["no_such_subcommand"], tmp_path).returncode == 106


def _declared(path):
    """Uncommented add_option / add_flag / add_subcommand names of a driver, in order."""
    names = {"option": [], "flag": [], "subcommand": []}
    for line in open(path, encoding="utf-8", errors="replace"):
        if line.lstrip().startswith("//"):
            continue
        for kind, name in re.findall(r'add_(option|flag|subcommand)\("([^"]+)"', line):
            names[kind].append(name)
    return names


def test_flag_lists_match_the_reference_sources():
    from oracle.oracle import REF_ROOT
    if not os.path.isdir(REF_ROOT):
        pytest.skip("reference sources not present on this machine")
    for exe, (rel, opts, flags) in DRIVERS.items():
        d = _declared(os.path.join(REF_ROOT, rel))
        assert sorted(d["option"]) == sorted(opts), exe
        assert sorted(d["flag"]) == sorted(flags), exe
    d = _declared(os.path.join(REF_ROOT, FMTCONV[0]))
    assert d["subcommand"] == FMTCONV[1]
    assert sorted(set(d["option"])) == sorted(FMTCONV[2])
