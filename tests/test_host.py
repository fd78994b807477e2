"""Host-side logic that needs no GPU: the C-ABI signatures the ctypes layer binds, the CTA work
splits and tile tables handed to the kernels, and the serving allocator."""

import re
from pathlib import Path

import numpy as np
import pytest
import torch

ROOT = Path(__file__).resolve().parent.parent


def header_declarations():
    """name -> (return type, [parameter types]) for every pe_* function in the header."""
    text = (ROOT / "include" / "pe_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    out = {}
    for ret, name, params in re.findall(r"\b((?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**)\s*(pe_[a-z0-9_]+)\s*\(([^)]*)\)\s*;",
                                        text):
        params = " ".join(params.split())
        types = [] if params in ("", "void") else [p.strip() for p in params.split(",")]
        out[name] = (ret.strip(), types)
    return out


def ctypes_kind(c_type):
    """The ctypes class a C parameter must be bound with (pointer types and streams as void*)."""
    import ctypes
    decl = c_type.replace("const ", "").strip()
    if "*" in decl or decl.split()[0] == "cudaStream_t":
        return ctypes.c_void_p
    base = decl.split()[0]
    return {"int64_t": ctypes.c_int64, "int": ctypes.c_int, "int32_t": ctypes.c_int, "double": ctypes.c_double}[base]


def test_ctypes_signatures_match_the_header():
    from panoptic_evaluator_gb300 import _native
    decls = header_declarations()
    assert set(_native.SIGNATURES) <= set(decls)
    for name, argtypes in _native.SIGNATURES.items():
        ret, params = decls[name]
        assert len(params) == len(argtypes), name
        for i, (c_type, bound) in enumerate(zip(params, argtypes)):
            assert ctypes_kind(c_type) is bound, f"{name} argument {i}: {c_type}"
        expected = "int64_t" if name in _native.INT64_RESULTS else "int"
        assert ret == expected, name


@pytest.fixture(scope="module")
def native_library():
    """The C-ABI library, built if needed (host entry points such as pe_contract_blocks run without a GPU)."""
    from panoptic_evaluator_gb300 import build
    return build.build()


def _check_bounds(bounds, total, ctas):
    assert bounds[0] == 0 and bounds[-1] == total
    assert len(bounds) == min(max(1, ctas), max(total, 1)) + 1
    assert np.all(np.diff(bounds) >= 0)


@pytest.mark.parametrize("seed", range(4))
def test_pass_bounds_split_bytes_evenly(seed):
    from panoptic_evaluator_gb300._batch import SEG_CHUNK, pass_bounds
    rng = np.random.default_rng(seed)
    B = int(rng.integers(1, 300))
    pixels = rng.integers(0, 1024 * 1024, B)
    pixels[rng.random(B) < 0.1] = 0
    dets = rng.integers(0, 100, B)
    ctas = int(rng.integers(1, 400))
    bounds = pass_bounds(pixels, dets, ctas)
    chunks = -(-pixels // SEG_CHUNK)
    total = int(chunks.sum())
    _check_bounds(bounds, total, ctas)
    # Cost of each chunk in bytes; no CTA exceeds the mean by more than one chunk.
    cost = np.concatenate([np.full(c, 8 + d) * np.minimum(SEG_CHUNK, p - SEG_CHUNK * np.arange(c))
                           for p, d, c in zip(pixels, dets, chunks)]) if total else np.zeros(0)
    per_cta = np.add.reduceat(cost, bounds[:-1]) * (np.diff(bounds) > 0) if total else np.zeros(0)
    if total:
        assert per_cta.sum() == cost.sum()
        assert per_cta.max() <= cost.sum() / len(per_cta) + cost.max()


def test_pass_bounds_edge_cases():
    from panoptic_evaluator_gb300._batch import pass_bounds
    assert list(pass_bounds([0, 0], [3, 4], 10)) == [0, 0]
    assert list(pass_bounds([5], [0], 10)) == [0, 1]
    b = pass_bounds([8192 * 3], [1], 100)
    assert list(b) == [0, 1, 2, 3]


@pytest.mark.parametrize("seed", range(4))
def test_contract_blocks_cover_every_pair_once(seed, native_library):
    from panoptic_evaluator_gb300._batch import CONTRACT_CHUNK, CONTRACT_ROWS, contract_blocks
    rng = np.random.default_rng(100 + seed)
    B = int(rng.integers(1, 40))
    dets = rng.integers(0, 300, B)
    gts = rng.integers(0, 140, B)
    pixels = rng.integers(0, 700 * 700, B)
    dets[0], gts[0] = 0, 5  # targets only
    table, total, bounds = contract_blocks(dets, gts, pixels, ctas=int(rng.integers(1, 200)))
    rows_a, rows_b = CONTRACT_ROWS
    seen = {}
    for image, m0, n0, first in table:
        assert m0 % rows_a == 0 and n0 % rows_b == 0
        assert m0 < max(dets[image], 1) and n0 < max(gts[image], 1)
        seen.setdefault(int(image), []).append((int(m0), int(n0), int(first)))
    for b in range(B):
        live = pixels[b] > 0 and (dets[b] > 0 or gts[b] > 0)
        if not live:
            assert b not in seen
            continue
        tiles = seen[b]
        m_tiles, n_tiles = max(-(-dets[b] // rows_a), 1), max(-(-gts[b] // rows_b), 1)
        assert sorted((m, n) for m, n, _ in tiles) == [(m * rows_a, n * rows_b) for m in range(m_tiles)
                                                          for n in range(n_tiles)]
    # Chunks are numbered tile after tile without gaps, each tile covering ceil(pixels / 4096) chunks.
    chunks = -(-pixels[table[:, 0]] // CONTRACT_CHUNK)
    assert list(table[:, 3]) == list(np.cumsum(chunks) - chunks)
    assert total == int(chunks.sum())
    _check_bounds(bounds, total, len(bounds) - 1)


@pytest.mark.parametrize("seed", range(3))
def test_contract_blocks_put_tma_images_after_staged(seed, native_library):
    """TMA images' blocks follow every staged image's blocks in chunk order, whatever the image order."""
    from panoptic_evaluator_gb300._batch import contract_blocks
    rng = np.random.default_rng(200 + seed)
    B = int(rng.integers(2, 30))
    dets, gts = rng.integers(0, 300, B), rng.integers(0, 140, B)
    pixels = rng.integers(1, 700 * 700, B)
    tma = rng.random(B) < 0.5
    table, total, bounds = contract_blocks(dets, gts, pixels, ctas=int(rng.integers(1, 200)), tma=tma)
    kinds = tma[table[:, 0]]
    assert not np.any(kinds[:-1] & ~kinds[1:]), "a staged block after a TMA block"
    plain, plain_total = contract_blocks(dets, gts, pixels)
    assert total == plain_total
    assert sorted(map(tuple, table[:, :3])) == sorted(map(tuple, plain[:, :3]))


@pytest.mark.parametrize("seed", range(4))
def test_contract_bounds_balance_chunk_costs(seed, native_library):
    """Each CTA range of pe_contract_blocks costs at most an even share plus one chunk.

    A chunk of block k costs its pixels x (the block's detection and target rows + 8), times the TMA weight
    for TMA images; the ranges are contiguous and every boundary follows the first chunk reaching i / R of
    the total.
    """
    from panoptic_evaluator_gb300._batch import CONTRACT_CHUNK, CONTRACT_ROWS, contract_blocks
    rng = np.random.default_rng(300 + seed)
    B = int(rng.integers(1, 50))
    dets, gts = rng.integers(0, 300, B), rng.integers(0, 140, B)
    pixels = rng.integers(1, 900 * 900, B)
    tma = rng.random(B) < 0.5
    weight_tma = float(rng.choice([0.45, 0.73, 1.2]))
    ctas = int(rng.integers(1, 300))
    table, total, bounds = contract_blocks(dets, gts, pixels, ctas=ctas, tma=tma, tma_cost=weight_tma)
    _check_bounds(bounds, total, ctas)
    rows_a, rows_b = CONTRACT_ROWS
    cost = []
    for image, m0, n0, _ in table:
        rows = min(rows_a, dets[image] - m0) + min(rows_b, gts[image] - n0) + 8
        w = (weight_tma if tma[image] else 1.0) * rows
        full, last = divmod(int(pixels[image]), CONTRACT_CHUNK)
        cost += [w * CONTRACT_CHUNK] * full + ([w * last] if last else [])
    cost = np.array(cost)
    assert len(cost) == total
    share = cost.sum() / (len(bounds) - 1)
    for lo, hi in zip(bounds[:-1], bounds[1:]):
        assert cost[lo:hi].sum() <= share + cost.max() * (1 + 1e-9)


def test_mask_flags_mark_row_alignment():
    """Bit 1: every mask row on a 16-byte boundary (both bases and H x W multiples of 16)."""
    from panoptic_evaluator_gb300.instance import mask_flags
    flags = mask_flags([0, 4096, 4100, 4096, 4112], [512, 512, 512, 516, 512], [4096, 420, 4096, 64, 4096])
    np.testing.assert_array_equal(flags, [2, 0, 0, 0, 2])


def test_arena_first_fit_coalesces():
    from panoptic_evaluator_gb300.serving import ALIGN, _Arena
    arena = _Arena(16 * ALIGN, "cpu")
    a = arena.allocate(1)
    b = arena.allocate(3 * ALIGN)
    c = arena.allocate(ALIGN + 1)
    assert (a, b, c) == (0, ALIGN, 4 * ALIGN)
    assert all(off % ALIGN == 0 for off in (a, b, c))
    assert arena.used == 6 * ALIGN and arena.largest() == 10 * ALIGN
    assert arena.allocate(11 * ALIGN) is None
    arena.release(b, 3 * ALIGN)
    assert arena.largest() == 10 * ALIGN  # the hole of 3 is not adjacent to the tail
    arena.release(a, 1)
    arena.release(c, ALIGN + 1)
    assert arena.free == [(0, 16 * ALIGN)] and arena.used == 0
    assert arena.allocate(16 * ALIGN) == 0 and arena.allocate(1) is None


def test_layout_views_are_aligned_and_disjoint():
    from panoptic_evaluator_gb300.serving import ALIGN, _Layout
    layout = _Layout()
    layout.add("a", 10)
    layout.add("b", 8 * 5)
    layout.add("c", 3)
    region = torch.zeros(layout.size, dtype=torch.uint8)
    offsets = [layout.parts[k][0] for k in ("a", "b", "c")]
    assert all(o % ALIGN == 0 for o in offsets) and offsets == sorted(offsets)
    b = layout.view(region, "b", torch.int64, (5,))
    b.fill_(-1)
    assert int(region[: offsets[1]].sum()) == 0 and int(region[offsets[2]:].sum()) == 0
    assert int(region[offsets[1]: offsets[1] + 40].sum()) == 40 * 255


def test_prefix_results_are_views_of_their_rows():
    from panoptic_evaluator_gb300 import prefix
    R, C, T = 6, 4, 2
    out = {k: torch.arange(R * C, dtype=torch.float64).reshape(R, C) + 1000 * i
           for i, k in enumerate(("tp", "fp", "fn", "sums"))}
    out["confusion"] = torch.arange(R * C * (C + 1), dtype=torch.int64).reshape(R, C, C + 1)
    for i, k in enumerate(("itp", "ifp", "ifn", "precision", "recall")):
        out[k] = torch.arange(R * T * C, dtype=torch.float64).reshape(R, T, C) + 100 * i
    out["values"] = torch.arange(R * 4 * C, dtype=torch.float64).reshape(R, 4, C)
    out["summaries"] = torch.arange(R * 9, dtype=torch.float64).reshape(R, 3, 3)
    out["counts"] = torch.arange(R * 3, dtype=torch.int64).reshape(R, 3)
    out["miou"] = torch.arange(R, dtype=torch.float64)
    thr = torch.tensor([0.5, 0.75], dtype=torch.float64)
    got = prefix.unpack(out, 2, [0, 5, 9], thr)
    assert not got[0]._cache  # nothing is materialised before it is read
    assert set(got[0]) == {"All", "Things", "Stuff", "prefix", "miou", "tp", "fp", "fn", "iou_sum", "confusion",
                           "per_class", "instance"} and len(got[0]) == 12
    assert [g["prefix"] for g in got] == [0, 5, 9]
    for offset, g in enumerate(got):
        r = 2 + offset
        assert torch.equal(g["tp"], out["tp"][r]) and torch.equal(g["confusion"], out["confusion"][r])
        assert g["miou"].item() == out["miou"][r].item()
        for i, name in enumerate(("All", "Things", "Stuff")):
            assert [g[name][k].item() for k in ("pq", "sq", "rq")] == out["summaries"][r, i].tolist()
            assert g[name]["n"].item() == out["counts"][r, i].item()
        assert torch.equal(g["per_class"]["iou"], out["values"][r, 3])
        assert torch.equal(g["instance"]["precision"], out["precision"][r])
        assert g["instance"]["iou_thresholds"] is thr
    # Views share storage with the outputs (no per-row copies), and a key read twice gives the same object.
    assert got[0]["tp"].data_ptr() == out["tp"][2].data_ptr()
    assert got[0]["All"] is got[0]["All"]
    assert dict(got[1])["prefix"] == 5


def test_admission_marks_requests_running_once_and_skips_cancelled():
    from concurrent.futures import Future

    from panoptic_evaluator_gb300.serving import _admitted

    class Job:
        def __init__(self):
            self.future = Future()

    queued, cancelled = Job(), Job()
    assert cancelled.future.cancel()
    assert _admitted(queued) and queued.future.running()
    assert _admitted(queued)  # put back after admission: still admitted, no second state change
    assert not queued.future.cancel()  # running requests cannot be cancelled
    assert not _admitted(cancelled) and cancelled.future.cancelled()


def test_gather_rows_pointers_and_element_sizes():
    """pe_inst_gather's rows: field pointers per image, size bits per field, None for dtypes it does not convert."""
    from panoptic_evaluator_gb300.instance import InstanceBatch, gather_rows
    masks = [torch.zeros((2, 4, 4), dtype=torch.bool), torch.zeros((3, 4, 4), dtype=torch.bool)]
    pc = [torch.tensor([1, 2], dtype=torch.int32), torch.tensor([3, 4, 5], dtype=torch.int64)]
    sc = [torch.tensor([0.5, 0.25], dtype=torch.float64), torch.tensor([0.1, 0.2, 0.3], dtype=torch.float32)]
    gc = [torch.tensor([7], dtype=torch.int64), torch.tensor([8, 9], dtype=torch.int32)]
    crowd = [torch.tensor([False]), torch.tensor([True, False])]
    areas = [torch.tensor([3.0], dtype=torch.float32), torch.tensor([4.0, 5.0], dtype=torch.float64)]
    pred = InstanceBatch(masks, pc, sc)
    target = InstanceBatch([torch.zeros((1, 4, 4), dtype=torch.bool), torch.zeros((2, 4, 4), dtype=torch.bool)], gc,
                           crowd=crowd, areas=areas)
    rows = gather_rows(pred, target, 2)
    assert rows.shape == (2, 6)
    for b in range(2):
        assert list(rows[b, :5]) == [pc[b].data_ptr(), sc[b].data_ptr(), gc[b].data_ptr(), crowd[b].data_ptr(),
                                     areas[b].data_ptr()]
    assert list(rows[:, 5]) == [2 | 4, 1 | 16]  # image 0: f64 scores, i64 gt classes; image 1: i64 classes, f64 areas
    no_crowd = gather_rows(pred, InstanceBatch(target.masks, gc), 2)
    assert list(no_crowd[:, 3]) == [0, 0] and list(no_crowd[:, 4]) == [0, 0]
    half = InstanceBatch(masks, pc, [s.to(torch.float16) for s in sc])
    assert gather_rows(half, target, 2) is None  # converted by torch instead
    strided = InstanceBatch(masks, [torch.tensor([1, 0, 2], dtype=torch.int32)[::2], pc[1]], sc)
    assert gather_rows(strided, target, 2) is None


def test_scratch_views_follow_size_and_dtype():
    """Scratch.get reuses a name's last view while size and dtype repeat, and re-slices after growth."""
    from panoptic_evaluator_gb300._batch import Scratch
    S = Scratch("cpu")
    a = S.get("x", 10, torch.int64)
    assert a.numel() == 10 and S.get("x", 10, torch.int64) is a
    grown = S.get("x", 20, torch.int64)
    assert grown.numel() == 20 and grown.data_ptr() != a.data_ptr()  # the buffer was reallocated
    again = S.get("x", 10, torch.int64)
    assert again.numel() == 10 and again.data_ptr() == grown.data_ptr()  # a view of the grown buffer
    other = S.get("x", 10, torch.int32)
    assert other.dtype == torch.int32 and other.numel() == 10
    zeroed = S.get("y", 4, torch.int32, zero=True)
    zeroed.fill_(7)
    assert int(S.get("y", 4, torch.int32, zero=True).sum()) == 0
    assert S.get("z", 0, torch.uint8).numel() == 1  # at least one element
