"""CPU-side checks of the C-ABI library: it loads, exports every declared symbol,
and its record layouts match the reference structs.  No compute calls (no GPU)."""
import ctypes as C

from gpu_index_test_gb300 import abi, native


def test_library_loads_and_exports_header_symbols():
    L = native.lib()
    syms = native.header_symbols()
    assert len(syms) >= 20
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing


def test_record_layouts():
    assert abi.REF_RANDSTROBE.itemsize == 16   # RefRandstrobe
    assert abi.QUERY_RANDSTROBE.itemsize == 24  # QueryRandstrobe
    assert abi.NAM.itemsize == 44               # Nam
    assert C.sizeof(abi.Params) == 48
    assert C.sizeof(abi.IndexInfo) == 64


def test_params_and_errors_without_gpu():
    p = native.params_from_read_length(150)
    assert (p.k, p.s, p.t_syncmer, p.w_min, p.w_max, p.q, p.max_dist) == (20, 16, 3, 5, 11, 255, 80)
    try:
        native.params_from_read_length(150, k=40)
    except native.GbsaError as e:
        assert e.code == abi.GBSA_ERR_PARAM
    else:
        raise AssertionError("k=40 accepted")
    # pick_bits (step2/index.cu:137-141): 5 Mbp → log2(1e6) - 1 = 18, 100 Mbp → 23
    assert native.lib().gbsa_pick_bits(C.byref(p), 5_000_000) == 18
    assert native.lib().gbsa_pick_bits(C.byref(p), 100_000_000) == 23
    assert native.lib().gbsa_pick_bits(C.byref(p), 3_100_000_000) == 28
    assert native.lib().gbsa_pick_bits(C.byref(p), 10) == 8


def test_batch_config_layout_and_default_without_gpu():
    """gbsa_batch_config is eight 32-bit fields; the default is the committed tuned file
    when it is present and well formed (no GPU needed to read it)."""
    import json
    import os

    assert C.sizeof(abi.BatchConfig) == 32
    cfg, from_file = native.batch_config_default()
    path = os.path.join(os.path.dirname(native.GBSA_SO), "tuned.json")
    if os.path.exists(path):
        assert from_file
        want = json.load(open(path))
        for k in ("seed_variant", "lane_max_hits", "sort_variant", "chunk_reads", "lane_variant", "warp_variant"):
            assert getattr(cfg, k) == want.get(k, 0), k
        assert cfg.rescue_block_hits == want.get("rescue_block_hits", 4000)
    else:
        assert not from_file
    assert 0 <= cfg.seed_variant < abi.SEED_VARIANTS and 1 <= cfg.lane_max_hits <= 160
