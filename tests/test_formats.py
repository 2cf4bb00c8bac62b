"""Edge-list formats and snapshot file checks (host only)."""
import numpy as np
import pytest


def test_binary_edge_list_round_trip(built_lib, tmp_path):
    import gpma_bfs_gb300 as G

    src, dst = G.gen_rmat(10, 8, seed=5)
    G.write_edges_bin(tmp_path / "g.bin", 1024, src, dst)
    n, s2, d2 = G.read_edges_bin(tmp_path / "g.bin")
    assert n == 1024 and np.array_equal(src, s2) and np.array_equal(dst, d2)
    # the text format holds the same graph
    G.write_edges_text(tmp_path / "g.txt", 1024, src, dst)
    n3, s3, d3 = G.read_edges_text(tmp_path / "g.txt")
    assert n3 == n and np.array_equal(s3, s2) and np.array_equal(d3, d2)
    # little-endian layout, whatever the host
    raw = (tmp_path / "g.bin").read_bytes()
    assert raw[:8] == b"GPMAEDG1" and int.from_bytes(raw[8:12], "little") == 1024
    assert int.from_bytes(raw[16:24], "little") == len(src)
    assert int.from_bytes(raw[24:28], "little") == int(src[0])


def test_binary_edge_list_rejects_bad_files(built_lib, tmp_path):
    import gpma_bfs_gb300 as G

    (tmp_path / "x.bin").write_bytes(b"not a graph")
    with pytest.raises(G.GPMAError):
        G.read_edges_bin(tmp_path / "x.bin")
    G.write_edges_bin(tmp_path / "t.bin", 8, np.arange(5, dtype=np.uint32), np.arange(5, dtype=np.uint32))
    data = (tmp_path / "t.bin").read_bytes()
    (tmp_path / "t.bin").write_bytes(data[:-3])  # truncated
    with pytest.raises(G.GPMAError):
        G.read_edges_bin(tmp_path / "t.bin")


def _snapshot_bytes(size=16, seg=2, height=3, row_num=2):
    """A well-formed snapshot header + payload of the given geometry (all
    slots empty) and its checksum, as gpma_save writes it."""
    payload = (b"\xff" * 8) * size + b"\x00" * size + b"\x00\x00\x00\x00" * (row_num + 1)
    h = 0x243F6A8885A308D3
    for byte in payload:
        h = ((h ^ byte) * 0x100000001B3) & 0xFFFFFFFFFFFFFFFF
        h ^= h >> 29
    hdr = (b"GPMASNP1" + (1).to_bytes(4, "little") + row_num.to_bytes(4, "little") + size.to_bytes(4, "little")
           + seg.to_bytes(4, "little") + height.to_bytes(4, "little") + bytes(4) + h.to_bytes(8, "little"))
    return hdr + payload


@pytest.mark.parametrize("mutate", ["magic", "truncate", "corrupt", "geometry", "trailing"])
def test_snapshot_load_rejects_before_touching_the_gpu(built_lib, tmp_path, mutate):
    import gpma_bfs_gb300 as G

    data = bytearray(_snapshot_bytes())
    if mutate == "magic":
        data[0:8] = b"GPMASNP9"
    elif mutate == "truncate":
        data = data[:-5]
    elif mutate == "corrupt":
        data[60] ^= 1
    elif mutate == "geometry":
        data = bytearray(_snapshot_bytes(size=16, seg=4, height=1))  # the reference would use segment 2
    else:
        data += b"\x00"
    p = tmp_path / "s.snap"
    p.write_bytes(bytes(data))
    with pytest.raises(G.GPMAError) as e:
        G.load(p)
    assert e.value.status == 6  # GPMA_ERR_IO


def test_oracle_side_generator_equals_the_library_generator(built_lib):
    """The CPU baselines build the benchmark graphs from the same generator
    source compiled on its own (oracle/_build/libgraphgen.so): same edges."""
    import gpma_bfs_gb300 as G
    from oracle.oracle import gen_chung_lu

    a = gen_chung_lu(20000, 300000, 2.3, 3000, 41)
    b = G.gen_chung_lu(20000, 300000, 2.3, 3000, 41)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
