"""Host side of the boundary (CPU only): loader, CSR builder, serialized cache,
JSON writer and generators, byte-checked against the reference's own loader
output in tests/golden/ (made by tests/golden/make_golden.py)."""
import os
import shutil

import numpy as np
import pytest

import kcoregpu_gb300 as kc
from conftest import GOLDEN, golden_core, golden_names, golden_serialized
from kcoregpu_gb300 import KCoreError


@pytest.mark.parametrize("name", golden_names(include_quirks=True))
def test_reference_mode_loader_matches_reference_csr(name):
    off, nbr, deg = kc.load_edgelist(str(GOLDEN / f"{name}.txt"), parse_mode="reference")
    roff, rnbr, rdeg = golden_serialized(name)
    np.testing.assert_array_equal(off, roff)
    np.testing.assert_array_equal(nbr, rnbr)
    np.testing.assert_array_equal(deg, rdeg)


@pytest.mark.parametrize("name", golden_names())
def test_snap_mode_loader_matches_reference_csr(name):
    off, nbr, deg = kc.load_edgelist(str(GOLDEN / f"{name}.txt"))
    roff, rnbr, _ = golden_serialized(name)
    np.testing.assert_array_equal(off, roff)
    np.testing.assert_array_equal(nbr, rnbr)


def test_snap_mode_skips_comment_and_blank_lines():
    # The reference turns '# ...' into edge (0, previous t) and a blank line into
    # a repeat of the previous edge (graph.cpp:86-88); SNAP mode skips them.
    off, nbr, _ = kc.load_edgelist(str(GOLDEN / "quirk_hash_blank.txt"))
    V = len(off) - 1
    assert V == 9
    adj = {v: nbr[off[v]:off[v + 1]].tolist() for v in range(V)}
    assert adj[0] == [] and adj[2] == [1]
    roff, rnbr, _ = golden_serialized("quirk_hash_blank")
    assert rnbr[roff[0]:roff[1]].tolist() == [2]   # the reference's injected edge


@pytest.mark.parametrize("name", golden_names(include_quirks=True))
def test_serialized_writer_bytes(name, tmp_path):
    off, nbr, deg = golden_serialized(name)
    out = tmp_path / "s.txt"
    kc.write_serialized(str(out), off, nbr, deg)
    assert out.read_bytes() == (GOLDEN / f"serialized-{name}.txt").read_bytes()


@pytest.mark.parametrize("name", golden_names(include_quirks=True))
def test_serialized_reader(name):
    off, nbr, deg = kc.read_serialized(str(GOLDEN / f"serialized-{name}.txt"))
    roff, rnbr, rdeg = golden_serialized(name)
    np.testing.assert_array_equal(off, roff)
    np.testing.assert_array_equal(nbr, rnbr)
    np.testing.assert_array_equal(deg, rdeg)


@pytest.mark.parametrize("name", golden_names(include_quirks=True))
def test_core_json_bytes(name, tmp_path):
    out = tmp_path / "j.txt"
    kc.write_core_json(str(out), golden_core(name))
    assert out.read_bytes() == (GOLDEN / f"pkc-kcore-{name}.txt").read_bytes()


def test_core_txt_format(tmp_path):
    out = tmp_path / "k-core.txt"
    kc.write_core_txt(str(out), np.array([0, 2, 2, 1], np.uint32))
    assert out.read_text() == "0 0\n1 2\n2 2\n3 1\n"


def test_graph_cache_roundtrip(tmp_path):
    # Graph(path): parse + write ./output/serialized-<basename>, then a second
    # construction reads the cache (graph.cpp:142-154).
    src = tmp_path / "g.txt"
    shutil.copy(GOLDEN / "skew_300.txt", src)
    outdir = tmp_path / "output"
    outdir.mkdir()
    g1 = kc.Graph(str(src), cache_dir=str(outdir))
    assert not g1.from_cache
    assert (outdir / "serialized-g.txt").read_bytes() == (GOLDEN / "serialized-skew_300.txt").read_bytes()
    g2 = kc.Graph(str(src), cache_dir=str(outdir))
    assert g2.from_cache and g2.cache_kind == 2      # the binary sidecar written beside it
    np.testing.assert_array_equal(g1.neighbors, g2.neighbors)
    np.testing.assert_array_equal(g1.neighbors_offset, g2.neighbors_offset)
    np.testing.assert_array_equal(g1.degrees, g2.degrees)
    assert g2.V == g1.V and g2.E == g1.E
    # a text cache rewritten after the sidecar wins over it (and refreshes it)
    side = outdir / "serialized-g.txt.kcb"
    os.utime(side, (1, 1))
    g3 = kc.Graph(str(src), cache_dir=str(outdir))
    assert g3.cache_kind == 1
    np.testing.assert_array_equal(g1.neighbors, g3.neighbors)
    assert kc.Graph(str(src), cache_dir=str(outdir)).cache_kind == 2


@pytest.mark.parametrize("name", ["k5", "skew_300"])
def test_binary_sidecar_roundtrip_and_rejects(name, tmp_path):
    off, nbr, deg = golden_serialized(name)
    p = tmp_path / "g.kcb"
    kc.write_csr_binary(str(p), off, nbr)
    o2, n2, d2 = kc.read_csr_binary(str(p))
    np.testing.assert_array_equal(o2, off)
    np.testing.assert_array_equal(n2, nbr)
    np.testing.assert_array_equal(d2, deg)
    raw = p.read_bytes()
    bad = tmp_path / "bad.kcb"
    for blob in (raw[:-4], raw + b"x", b"XXXXXXXX" + raw[8:]):   # truncated, trailing, magic
        bad.write_bytes(blob)
        with pytest.raises(KCoreError) as e:
            kc.read_csr_binary(str(bad))
        assert e.value.name == "KC_ERR_PARSE"
    # a neighbour id >= V
    arr = bytearray(raw)
    arr[-4:] = (len(off) + 7).to_bytes(4, "little")
    bad.write_bytes(bytes(arr))
    with pytest.raises(KCoreError):
        kc.read_csr_binary(str(bad))


def test_graph_cache_dir_missing_is_silent(tmp_path):
    src = tmp_path / "g.txt"
    shutil.copy(GOLDEN / "k5.txt", src)
    g = kc.Graph(str(src), cache_dir=str(tmp_path / "nope"))
    assert g.V == 5 and g.E == 20
    assert not (tmp_path / "nope").exists()


def test_build_csr_semantics():
    # self-loops dropped before V is computed; V = max id + 1; dedup; ascending
    off, nbr, deg = kc.build_csr([5, 1, 2, 2, 3], [5, 2, 1, 3, 1])
    assert len(off) - 1 == 4
    assert nbr[off[1]:off[2]].tolist() == [2, 3]
    assert deg.tolist() == [0, 2, 2, 2]
    off, nbr, deg = kc.build_csr([4], [4])          # only a self-loop
    assert len(off) == 2 and len(nbr) == 0          # V = 1 (graph.cpp:96)
    off, nbr, deg = kc.build_csr([], [])
    assert len(off) == 2


def test_loader_errors(tmp_path):
    with pytest.raises(KCoreError) as e:
        kc.load_edgelist(str(tmp_path / "missing.txt"))
    assert e.value.name == "KC_ERR_IO"
    bad = tmp_path / "bad.txt"
    bad.write_text("1 2\n3 x\n")
    with pytest.raises(KCoreError) as e:
        kc.load_edgelist(str(bad))
    assert e.value.name == "KC_ERR_PARSE"
    first = tmp_path / "first.txt"
    first.write_text("# header\n1 2\n")
    with pytest.raises(KCoreError) as e:       # undefined in the reference (t unset)
        kc.load_edgelist(str(first), parse_mode="reference")
    assert e.value.name == "KC_ERR_PARSE"
    assert len(kc.load_edgelist(str(first))[0]) == 4


def test_truncated_serialized_is_rejected(tmp_path):
    p = tmp_path / "serialized-x"
    data = (GOLDEN / "serialized-k5.txt").read_text()
    p.write_text(data[: len(data) // 2])
    with pytest.raises(KCoreError) as e:
        kc.read_serialized(str(p))
    assert e.value.name == "KC_ERR_PARSE"


def test_large_parallel_parse_matches_build(tmp_path):
    s, t = kc.gen_rmat(50000, 400000, seed=11)
    p = tmp_path / "big.txt"
    kc.write_edgelist(str(p), s, t)
    a = kc.load_edgelist(str(p))
    b = kc.load_edgelist(str(p), parse_mode="reference")
    c = kc.build_csr(s, t)
    for x, y, z in zip(a, b, c):
        np.testing.assert_array_equal(x, y)
        np.testing.assert_array_equal(x, z)


def test_generators_are_deterministic():
    a = kc.gen_rmat(4096, 20000, seed=5)
    b = kc.gen_rmat(4096, 20000, seed=5)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    assert a[0].max() < 4096 and a[1].max() < 4096
    c = kc.gen_chung_lu(5000, 12000, 2.1, 500.0, seed=3)
    d = kc.gen_chung_lu(5000, 12000, 2.1, 500.0, seed=3)
    np.testing.assert_array_equal(c[0], d[0])
    pairs = {(min(x, y), max(x, y)) for x, y in zip(c[0].tolist(), c[1].tolist())}
    assert len(pairs) == 12000 and all(x != y for x, y in pairs)
    e = kc.gen_er(1000, 3000, seed=9)
    assert len({(min(x, y), max(x, y)) for x, y in zip(e[0].tolist(), e[1].tolist())}) == 3000
