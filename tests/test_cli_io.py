"""The drop-in executables' own file readers and writers (nbpg_gb300/cli/common.h), compiled
into a small host program with g++ (no device work): a `.graph` file written by the
reference's Vamana binary (golden bytes) is read and rewritten byte for byte, vector files
are read with and without a row limit, and the ids of a `.gt` file come back as written."""
import os
import subprocess

import numpy as np
import pytest

from nbpg_gb300 import formats

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROG = r"""
#include <cstdio>
#include <cstring>
#include "common.h"
using namespace nbpg_cli;
int main(int argc, char **argv)
{
    const std::string mode = argv[1], in = argv[2], out = argv[3];
    if (mode == "graph") {
        uint32_t n, R;
        std::vector<uint32_t> g = read_graph(in, n, R);
        write_graph(out, g, n, R);
    } else if (mode == "rows") {
        uint32_t n, d;
        std::vector<uint8_t> v = read_rows(in, n, d, uint32_t(std::atoi(argv[4])));
        std::ofstream w(out, std::ios::binary);
        w.write(reinterpret_cast<const char *>(&n), 4);
        w.write(reinterpret_cast<const char *>(&d), 4);
        w.write(reinterpret_cast<const char *>(v.data()), v.size());
    } else if (mode == "gt") {
        uint32_t nq, k;
        std::vector<uint32_t> ids = read_gt_ids(in, nq, k);
        std::ofstream w(out, std::ios::binary);
        w.write(reinterpret_cast<const char *>(ids.data()), ids.size() * 4);
    } else {
        return 2;
    }
    return 0;
}
"""


@pytest.fixture(scope="module")
def prog(tmp_path_factory):
    d = tmp_path_factory.mktemp("cli_io")
    src, exe = d / "io.cpp", d / "io"
    src.write_text(PROG)
    cli = os.path.join(ROOT, "nbpg_gb300", "cli")
    r = subprocess.run(["g++", "-O1", "-std=c++17", f"-I{cli}", f"-I{os.path.join(ROOT, 'include')}", str(src), "-o",
                        str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return str(exe)


def _run(prog, *args):
    r = subprocess.run([prog, *map(str, args)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr


@pytest.mark.parametrize("name", ["graph_vamana.npz", "graph_split1_dyn.npz", "fgim_split4.npz"])
def test_graph_file_round_trip(prog, tmp_path, name):
    raw = np.load(os.path.join(ROOT, "tests", "golden", name))["graph_file"].tobytes()
    (tmp_path / "in.graph").write_bytes(raw)
    _run(prog, "graph", tmp_path / "in.graph", tmp_path / "out.graph")
    assert (tmp_path / "out.graph").read_bytes() == raw


def test_vector_rows_with_limit(prog, tmp_path):
    x = np.random.default_rng(2).integers(0, 256, (23, 40)).astype(np.uint8)
    formats.write_vectors(str(tmp_path / "x.u8bin"), x)
    for limit in (0, 7, 50):
        _run(prog, "rows", tmp_path / "x.u8bin", tmp_path / "o.u8bin", limit)
        want = x if limit in (0, 50) else x[:limit]
        assert np.array_equal(formats.read_vectors(str(tmp_path / "o.u8bin")), want), limit


def test_gt_ids(prog, tmp_path):
    r = np.random.default_rng(4)
    ids = r.integers(0, 1 << 20, (9, 12)).astype(np.uint32)
    formats.write_gt(str(tmp_path / "a.gt"), ids, r.random((9, 12)).astype(np.float32))
    _run(prog, "gt", tmp_path / "a.gt", tmp_path / "ids.bin")
    assert np.array_equal(np.fromfile(str(tmp_path / "ids.bin"), np.uint32).reshape(9, 12), ids)
