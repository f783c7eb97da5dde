#!/usr/bin/env python3
"""Generate golden vectors from the reference's own code (run where its sources exist).

Inputs are small seeded synthetic sets.  Outputs, stored as tests/golden/*.npz:
  * gt_*.npz      CompGT binary output (.gt ids/dists), k=100, u8/i8, L2 and --use_mips,
                  including a tie-heavy set where CompGT's stale read matters;
  * graph_*.npz   .graph files written by the Vamana binary with deterministic settings
                  (--num_split 0, and --num_split 1 which runs the split stage, a popularity
                  pass and the dynamic-prune pass), kept as raw bytes;
  * search_*.npz  per-query ids, dists, counts, expansions and distance counts from the
                  harness over the reference headers (qsearchAll's body) on those graphs;
  * pca.npz       PCACompress outputs (.u4bin/.i4bin/.u8bin/.i8bin/.fbin) for float rows and
                  a .mat with bias; for u8/i8 input rows (whose path in the reference only
                  works on whole 100,000-row blocks) the seed of the rows and the SHA-256 of
                  the reference's output instead of the rows themselves;
  * fmtconv.npz   FmtConv fbin2u8bin, u8bin2u4bin (odd row length) and vec2bin outputs;
  * fgim_*.npz    .graph files written by the FGIM binary (pair passes, split stage, dynamic
                  prune, rand_sp), kept as raw bytes;
  * rerank_*.npz  beam_search_rerank through the harness with raw float rows beside 4-bit
                  (L2) and u8 (inner product) quantised rows: rerank factors 100, 3 and 0
                  (filtering mode), on a graph built by the oracle.

Usage: make -C oracle ref && python tests/golden/make_golden.py [--only pca,rerank,fgim,hnsw]
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from nbpg_gb300 import formats, synth  # noqa: E402
from oracle.oracle import REF_COMPGT, REF_VAMANA, reference  # noqa: E402

REF_DIR = os.path.dirname(REF_COMPGT)


def pca_rows_u8in(seed):
    """Rows for the u8/i8-input PCACompress pins: 100,000 x 48 (one reference block)."""
    r = np.random.default_rng(seed)
    return r.integers(0, 256, (100000, 48)).astype(np.uint8), r.integers(-128, 128, (100000, 48)).astype(np.int8)


def pca_golden(tmp):
    import hashlib
    r = np.random.default_rng(13)
    x = (r.normal(size=(600, 32)) * 0.6).astype(np.float32)
    mat = (r.normal(size=(16, 32)) * 0.3).astype(np.float32)
    bias = (r.normal(size=16) * 0.1).astype(np.float32)
    formats.write_vectors(f"{tmp}/x.fbin", x)
    formats.write_matrix(f"{tmp}/m.mat", mat, bias)
    out = {"x": x, "mat": mat, "bias": bias}
    for kind, ext in [("u4", ".u4bin"), ("i4", ".i4bin"), ("u8", ".u8bin"), ("i8", ".i8bin"), ("f32", ".fbin")]:
        subprocess.run([f"{REF_DIR}/PCACompress", "--ifile", f"{tmp}/x.fbin", "--ofile", f"{tmp}/o{ext}", "--matFile",
                        f"{tmp}/m.mat"], check=True, stdout=subprocess.DEVNULL)
        out["out_" + kind] = np.fromfile(f"{tmp}/o{ext}", dtype=np.uint8)
    m2 = (r.normal(size=(16, 48)) * 0.3 / 200).astype(np.float32)
    formats.write_matrix(f"{tmp}/m2.mat", m2, bias)
    xu, xi = pca_rows_u8in(29)
    for name, rows, ext in [("u8in", xu, ".u8bin"), ("i8in", xi, ".i8bin")]:
        formats.write_vectors(f"{tmp}/r{ext}", rows)
        subprocess.run([f"{REF_DIR}/PCACompress", "--ifile", f"{tmp}/r{ext}", "--ofile", f"{tmp}/r_{name}.u4bin",
                        "--matFile", f"{tmp}/m2.mat"], check=True, stdout=subprocess.DEVNULL)
        out["sha_" + name] = np.array(hashlib.sha256(open(f"{tmp}/r_{name}.u4bin", "rb").read()).hexdigest())
    out["mat_u8in"] = m2
    out["seed_u8in"] = np.array(29)
    np.savez_compressed(f"{HERE}/pca.npz", **out)

    xf = r.uniform(0, 255.99, (300, 24)).astype(np.float32)
    formats.write_vectors(f"{tmp}/f.fbin", xf)
    subprocess.run([f"{REF_DIR}/FmtConv", "fbin2u8bin", "--ifile", f"{tmp}/f.fbin", "--ofile", f"{tmp}/f.u8bin"],
                   check=True, stdout=subprocess.DEVNULL)
    xu8 = r.integers(0, 256, (300, 25)).astype(np.uint8)
    formats.write_vectors(f"{tmp}/g.u8bin", xu8)
    subprocess.run([f"{REF_DIR}/FmtConv", "u8bin2u4bin", "--ifile", f"{tmp}/g.u8bin", "--ofile", f"{tmp}/g.u4bin"],
                   check=True, stdout=subprocess.DEVNULL)
    formats.write_fvecs(f"{tmp}/v.fvecs", xf[:40])
    subprocess.run([f"{REF_DIR}/FmtConv", "vec2bin", "--ifile", f"{tmp}/v.fvecs", "--ofile", f"{tmp}/v.fbin"],
                   check=True, stdout=subprocess.DEVNULL)
    np.savez_compressed(f"{HERE}/fmtconv.npz", f32=xf, f32_to_u8=np.fromfile(f"{tmp}/f.u8bin", dtype=np.uint8),
                        u8=xu8, u8_to_u4=np.fromfile(f"{tmp}/g.u4bin", dtype=np.uint8),
                        fvecs=np.fromfile(f"{tmp}/v.fvecs", dtype=np.uint8),
                        vec2bin=np.fromfile(f"{tmp}/v.fbin", dtype=np.uint8))


def datasets():
    b, q = synth.u8_mixture(3000, 40, dim=32, n_centres=12, seed=7)
    r = np.random.default_rng(5)
    tb, tq = r.integers(0, 4, (2000, 8)).astype(np.uint8), r.integers(0, 4, (30, 8)).astype(np.uint8)
    ib, iq = synth.i8_unit_mixture(2500, 30, dim=24, n_centres=10, seed=3)
    return {"mix": ("u8", ".u8bin", b, q), "tie": ("u8", ".u8bin", tb, tq), "i8": ("i8", ".i8bin", ib, iq)}


def rerank_golden():
    from oracle.oracle import oracle
    ref = reference()
    r = np.random.default_rng(17)
    n, nq, d = 1500, 40, 16
    raw = r.normal(size=(n, d)).astype(np.float32)
    rq = r.normal(size=(nq, d)).astype(np.float32)
    cb = np.clip(np.round((raw + 3) * 40), 0, 255).astype(np.uint8)
    cq = np.clip(np.round((rq + 3) * 40), 0, 255).astype(np.uint8)
    for name, dtype, metric, qb, qq in [("u4_l2", "u4", "l2", synth.pack_u4(cb >> 4), synth.pack_u4(cq >> 4)),
                                        ("u8_ip", "u8", "ip", cb, cq)]:
        g, _, _, _ = oracle().build_graph(dtype, metric, qb, R=16, L=32, VL=48, num_split=0, num_passes=1)
        out = {"base": qb, "queries": qq, "raw": raw, "raw_queries": rq, "graph": g}
        for L, k, rf in [(32, 10, 100), (40, 5, 3), (32, 10, 0)]:
            ids, ds, cnt, vis, cmps = ref.search_rerank(dtype, metric, qb, raw, g, qq, rq, L, k, rf)
            out.update({f"ids_{L}_{k}_{rf}": ids, f"dists_{L}_{k}_{rf}": ds, f"count_{L}_{k}_{rf}": cnt,
                        f"visited_{L}_{k}_{rf}": vis, f"cmps_{L}_{k}_{rf}": cmps})
        np.savez_compressed(f"{HERE}/rerank_{name}.npz", **out)


def fgim_golden(tmp):
    b, _ = synth.u8_mixture(3000, 1, dim=32, n_centres=12, seed=7)
    formats.write_vectors(f"{tmp}/fb.u8bin", b)
    builds = {
        "split4": ["--num_split", "4", "--num_passes", "2"],
        "dyn3": ["--num_split", "4", "--num_passes", "3", "--dynamic_prune", "--min_alpha", "1.05", "--max_alpha",
                 "1.2"],
        "randsp": ["--num_split", "2", "--num_passes", "2", "--rand_sp"],
    }
    for name, flags in builds.items():
        ip = f"{tmp}/fidx_{name}"
        subprocess.run([os.path.join(REF_DIR, "FGIM"), "--quant_base_path", f"{tmp}/fb.u8bin", "--index_path", ip,
                        "--R", "16", "--L", "24", "--VL", "32", "--rebuild", *flags], check=True,
                       stdout=subprocess.DEVNULL)
        raw = open(ip + ".graph", "rb").read()
        np.savez_compressed(f"{HERE}/fgim_{name}.npz", base=b, graph_file=np.frombuffer(raw, np.uint8),
                            flags=np.array(" ".join(["--R 16 --L 24 --VL 32"] + flags)))


def hnsw_golden(tmp, ref):
    """.graph/.hid files written by the reference HNSW driver, the harness's per-node counters for
    the same build, its hier_qsearchAll results on 200 queries, and Prune::maxAnglePrune on
    candidate lists drawn from those builds."""
    b, q = synth.u8_mixture(3000, 200, dim=32, n_centres=12, seed=7)
    formats.write_vectors(f"{tmp}/hb.u8bin", b)
    builds = {
        "default": dict(flags=[], kw={}),
        "hb3": dict(flags=["--hier_beamSize", "3", "--m_l", "0.6", "--alpha", "1.2"],
                    kw=dict(hier_beam=3, m_l=0.6, alpha=1.2)),
        "pr": dict(flags=["--PR", "48", "--m_l", "6", "--max_node_num", "40000"], kw=dict(PR=48, m_l=6.0,
                                                                                        max_node=40000)),
    }
    for name, spec in builds.items():
        ip = f"{tmp}/hidx_{name}"
        subprocess.run([os.path.join(REF_DIR, "HNSW"), "--quant_base_path", f"{tmp}/hb.u8bin", "--index_path", ip,
                        "--R", "16", "--L", "24", "--VL", "48", "--rebuild", *spec["flags"]], check=True,
                       stdout=subprocess.DEVNULL)
        graph_raw = open(ip + ".graph", "rb").read()
        hid_raw = open(ip + ".hid", "rb").read()
        g, pre, sp, sv, sd, iso = ref.build_hnsw("u8", "l2", b, R=16, L=24, VL=48, **spec["kw"])
        hb = spec["kw"].get("hier_beam", 1)
        ids, cnt, vis, cm = ref.search_hnsw("u8", "l2", b, g, pre, sp, q, L=24, k=10, hier_beam=hb)
        np.savez_compressed(f"{HERE}/hnsw_{name}.npz", base=b, queries=q, graph_file=np.frombuffer(graph_raw, np.uint8),
                            hid_file=np.frombuffer(hid_raw, np.uint8), stat_visited=sv, stat_dist=sd, isolated=iso,
                            q_ids=ids, q_count=cnt, q_visited=vis, q_cmps=cm, hier_beam=hb,
                            flags=np.array(" ".join(["--R 16 --L 24 --VL 48"] + spec["flags"])))
    # maxAnglePrune on the visited-like lists of a search over the default build's level-0 rows
    r = np.random.default_rng(5)
    cases = []
    for t in range(60):
        p = int(r.integers(0, len(b)))
        m = int(r.integers(1, 48))
        cand = r.choice(np.delete(np.arange(len(b)), p), size=m, replace=False).astype(np.uint32)
        d = np.array([ref.distance("u8", "l2", b[p], b[c]) for c in cand], np.float32)
        o = np.lexsort((cand, d))
        cand, d = cand[o], d[o]
        alpha, cosa = [(1.2, 0.0), (1.0, 0.5), (1.1, 0.8), (0.0, 0.6)][t % 4]
        R = [8, 16, 32][t % 3]
        oi, od, oc = ref.max_angle_prune("u8", "l2", b, p, cand, d, R, 48, alpha, cosa)
        cases.append((p, cand, d, alpha, cosa, R, oi, od, oc))
    np.savez_compressed(f"{HERE}/max_angle_prune.npz", base=b,
                        p=np.array([c[0] for c in cases], np.uint32),
                        alpha=np.array([c[3] for c in cases]), cos=np.array([c[4] for c in cases]),
                        R=np.array([c[5] for c in cases], np.uint32),
                        cmps=np.array([c[8] for c in cases], np.uint32),
                        cand=np.array([np.pad(c[1], (0, 48 - len(c[1])), constant_values=0xFFFFFFFF) for c in cases]),
                        dist=np.array([np.pad(c[2], (0, 48 - len(c[2]))) for c in cases]),
                        n_cand=np.array([len(c[1]) for c in cases], np.uint32),
                        out=np.array([np.pad(c[6], (0, 48 - len(c[6])), constant_values=0xFFFFFFFF) for c in cases]),
                        out_d=np.array([np.pad(c[7], (0, 48 - len(c[7]))) for c in cases]),
                        n_out=np.array([len(c[6]) for c in cases], np.uint32))


def main():
    if not (os.path.exists(REF_COMPGT) and os.path.exists(REF_VAMANA) and reference()):
        sys.exit("build the reference first: make -C oracle ref")
    ref = reference()
    tmp = tempfile.mkdtemp()
    only = sys.argv[sys.argv.index("--only") + 1].split(",") if "--only" in sys.argv else None
    if only is None or "pca" in only:
        pca_golden(tmp)
    if only is None or "rerank" in only:
        rerank_golden()
    if only is None or "fgim" in only:
        fgim_golden(tmp)
    if only is None or "hnsw" in only:
        hnsw_golden(tmp, ref)
    if only is not None:
        print("golden vectors written to", HERE)
        return
    for name, (dt, ext, b, q) in datasets().items():
        bp, qp = f"{tmp}/{name}_b{ext}", f"{tmp}/{name}_q{ext}"
        formats.write_vectors(bp, b)
        formats.write_vectors(qp, q)
        for mips in (False, True):
            gp = f"{tmp}/{name}_{int(mips)}.gt"
            cmd = [REF_COMPGT, "--base_path", bp, "--query_path", qp, "--gt_path", gp, "--k", "100"]
            if mips:
                cmd.append("--use_mips")
            subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL)
            ids, ds = formats.read_gt(gp)
            np.savez_compressed(f"{HERE}/gt_{name}_{'ip' if mips else 'l2'}.npz", base=b, queries=q, ids=ids,
                                dists=ds, dtype=dt)

    dt, ext, b, q = datasets()["mix"]
    bp = f"{tmp}/g_base{ext}"
    formats.write_vectors(bp, b)
    builds = {
        "vamana": ["--num_split", "0", "--num_passes", "1", "--max_alpha", "1.2"],
        "split1_dyn": ["--num_split", "1", "--num_passes", "2", "--dynamic_prune", "--min_alpha", "1.05",
                       "--max_alpha", "1.2"],
    }
    for name, flags in builds.items():
        ip = f"{tmp}/idx_{name}"
        subprocess.run([REF_VAMANA, "--quant_base_path", bp, "--index_path", ip, "--R", "16", "--L", "24", "--VL",
                        "32", "--rebuild", *flags], check=True, stdout=subprocess.DEVNULL)
        raw = open(ip + ".graph", "rb").read()
        np.savez_compressed(f"{HERE}/graph_{name}.npz", base=b, graph_file=np.frombuffer(raw, np.uint8),
                            flags=np.array(" ".join(["--R 16 --L 24 --VL 32"] + flags)))
        g = formats.read_graph(ip + ".graph")
        for L, k in [(10, 10), (32, 10), (64, 50)]:
            out = ref.search("u8", "l2", b, g, q, L=L, k=k, cut=1.35)
            np.savez_compressed(f"{HERE}/search_{name}_L{L}_k{k}.npz", ids=out[0], dists=out[1], count=out[2],
                                visited=out[3], cmps=out[4], queries=q)
    print("golden vectors written to", HERE)


if __name__ == "__main__":
    main()
