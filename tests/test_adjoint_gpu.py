"""Adjoint (pga_adjoint / torch.autograd) against FP64 central differences.

The derivation tree is frozen by the forward pass.  For a linear loss
L = sum(W * M) over the terminal transforms (W random, matched to terminals by
derivation-path hash) the gradient with respect to the per-axiom parameter
blocks and the axiom sizes is compared with central finite differences
(h = 1e-4) of the oracle's double-precision derivation.  Perturbations that
change the set of derivation paths (a branch or a repetition count flips) are
skipped: the derivative is only defined away from those boundaries.
Tolerance: FP32 forward and adjoint against FP64 differences, relative 2e-3 of
the gradient's scale.
"""
import numpy as np
import pytest

import oracle
from operatorgraph_gb300 import grammar as G
from operatorgraph_gb300 import scenes

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

H = 1e-4
RTOL = 2e-3


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from operatorgraph_gb300 import build as B

    B.build()
    torch.cuda.set_device(0)


def _loss64(batch, weights_by_path, blocks64=None, sizes64=None):
    """sum over terminals of W . M in FP64 (oracle) and the set of derivation paths."""
    M, P = oracle.derive_f64(G.DEFAULT_PROCS, batch["entries"], batch["axioms"], blocks64, batch["block_stride"],
                             sizes64)
    total, keys = 0.0, []
    for m, p in zip(M, P):
        w = weights_by_path.get(int(p))
        if w is None:
            return None, None
        total += float(np.dot(w, m))
        keys.append(int(p))
    return total, frozenset(keys)


def _gpu_grad(batch, weights_seed=3):
    from operatorgraph_gb300.autograd import axioms_tensor, derive_transforms
    from operatorgraph_gb300.engine import Engine

    n_ref = len(oracle.derive(G.DEFAULT_PROCS, batch["entries"], batch["axioms"], batch["blocks"],
                              batch["block_stride"]))
    eng = Engine(batch["entries"], block_stride=batch["block_stride"], record_tape=True, node_capacity=1 << 20,
                 max_terminals=1 << 20)
    d_ax = axioms_tensor(batch["axioms"])
    blocks = None
    if batch["blocks"] is not None:
        blocks = torch.tensor(batch["blocks"], dtype=torch.float32, device="cuda", requires_grad=True)
    sizes = torch.tensor(batch["axioms"]["size"], dtype=torch.float32, device="cuda", requires_grad=True)
    M, paths = derive_transforms(eng, d_ax, blocks, sizes, n_ref)
    assert M.shape[0] == n_ref
    rng = np.random.default_rng(weights_seed)
    W = rng.standard_normal((n_ref, 12))
    loss = (M * torch.tensor(W, dtype=torch.float32, device="cuda")).sum()
    loss.backward()
    by_path = {int(p): W[i] for i, p in enumerate(paths.cpu().numpy().view(np.uint64))}
    gb = None if blocks is None else blocks.grad.detach().cpu().numpy().astype(np.float64)
    gs = sizes.grad.detach().cpu().numpy().astype(np.float64)
    eng.release()
    return by_path, gb, gs


def _central(batch, by_path, keys0, base, b64, s64, perturb):
    """(central difference, forward difference, backward difference) or None
    when the perturbation changes the set of derivation paths."""
    bp, sp = perturb(b64, s64, +H)
    bm, sm = perturb(b64, s64, -H)
    lp, kp = _loss64(batch, by_path, bp, sp)
    lm, km = _loss64(batch, by_path, bm, sm)
    if lp is None or lm is None or kp != keys0 or km != keys0:
        return None  # a branch, a repetition count or a discard flips within +-H
    return (lp - lm) / (2 * H), (lp - base) / H, (base - lm) / H


def _compare(label, got, diffs):
    """Checks every smooth entry of diffs (None: skipped); returns how many.

    An input sitting on a kink (an exact Repeat division, where the remainder
    piece switches between zero and a full extent while the extra piece is
    discarded) keeps its path set but has different one-sided slopes: the
    central difference is no derivative there, so entries whose forward and
    backward differences disagree are skipped too."""
    fds = [d[0] for d in diffs if d is not None]
    scale = max(max((abs(f) for f in fds), default=0.0), 1.0)
    checked = 0
    for k, d in enumerate(diffs):
        if d is None or abs(d[1] - d[2]) > 0.5 * RTOL * scale:
            continue
        _check(f"{label}[{k}]", got[k], d[0], scale)
        checked += 1
    return checked


def _check(name, got, fd, scale):
    err = abs(got - fd)
    assert err <= RTOL * scale + 1e-6, f"{name}: adjoint {got:.6g} vs FD {fd:.6g} (scale {scale:.3g})"


def test_facade_block_and_size_gradients_match_fp64_central_differences():
    batch = scenes.facades(8, seed=7)
    by_path, gb, gs = _gpu_grad(batch)
    b64 = batch["blocks"].astype(np.float64)
    s64 = batch["axioms"]["size"].astype(np.float64)
    base, keys0 = _loss64(batch, by_path, b64, s64)
    assert base is not None and len(keys0) == len(by_path)

    def block_at(k):
        def f(b, s, h):
            b = b.copy()
            b[k] += h
            return b, s
        return f

    def size_at(k):
        def f(b, s, h):
            s = s.copy()
            s.reshape(-1)[k] += h
            return b, s
        return f

    diffs = [_central(batch, by_path, keys0, base, b64, s64, block_at(k)) for k in range(len(b64))]
    assert _compare("block", gb, diffs) >= len(b64) * 0.9
    diffs = [_central(batch, by_path, keys0, base, b64, s64, size_at(k)) for k in range(s64.size)]
    assert _compare("size", gs.reshape(-1), diffs) == s64.size


def _size_cases():
    import sys
    from pathlib import Path

    sys.path.insert(0, str(Path(__file__).parent / "golden"))
    import cases as C

    # every golden case, Rotate ones included (the general-frame build's adjoint)
    out = list(C.cases())
    for mode in (G.ANCHOR_TO_START, G.ANCHOR_TO_END, G.ADJUST_TO_FILL):
        out.append((f"building_off_grid_m{mode}", scenes.building(w=25.3, d=19.7, h=31.0, mode=mode)))
    out.append(("forest_2", scenes.forest(2)))
    return out


_SIZE_CASES = _size_cases()


@pytest.mark.parametrize("name,batch", _SIZE_CASES, ids=[c[0] for c in _SIZE_CASES])
def test_axiom_size_gradients_match_fp64_central_differences(name, batch):
    """Every operator's VJP through the axiom sizes: Subdivide (static, dynamic,
    absolute / relative / zero factors), Repeat (three modes, relative and
    absolute extents), ComponentSplit, Extrude, IfSizeLess chains, and with
    Rotate at arbitrary angles (the general-frame kernels: the turned frame
    carries the translation and size gradients), Replicate, Translate, Scale."""
    by_path, _, gs = _gpu_grad(batch)
    b64 = None if batch["blocks"] is None else batch["blocks"].astype(np.float64)
    s64 = batch["axioms"]["size"].astype(np.float64)
    base, keys0 = _loss64(batch, by_path, b64, s64)
    assert base is not None and len(keys0) == len(by_path)

    def size_at(k):
        def f(b, s, h):
            s = s.copy()
            s.reshape(-1)[k] += h
            return b, s
        return f

    diffs = [_central(batch, by_path, keys0, base, b64, s64, size_at(k)) for k in range(s64.size)]
    checked = _compare(name, gs.reshape(-1), diffs)
    if checked == 0:
        pytest.skip("every axiom size sits on a kink or a discrete boundary")


def _affine_blocks_batch(n=6, seed=5):
    """Translate and Scale driven by per-axiom blocks: a RandomRule on the seed
    picks a translated-and-scaled box (relative x, absolute y, expression z
    translate) or its faces, each replicated into an extruded, translated box
    and the face itself, so both smooth-step kinds, the discrete choice and
    Replicate sit between the inputs and the terminals."""
    from operatorgraph_gb300.grammar import DispatchTable, Entry, block, scalar, shape_attr

    tab = DispatchTable([
        Entry(G.BOX_RANDOM_RULE, [shape_attr(15), scalar(0.5), scalar(0.5)], [(1, 0), (4, 0)]),
        Entry(G.BOX_TRANSLATE, [block(0), block(1), G.exp(("a", 13), ("s", 0.25), ("op", G.OPT_MULTI))], [(2, 0)]),
        Entry(G.BOX_SCALE, [block(2), block(3), scalar(-1)], [(3, 0)]),
        Entry(G.BOX_GENERATE, [scalar(0)], []),
        Entry(G.BOX_COMPONENT_SPLIT, [], [(5, 0), (8, 0), (5, 0)]),
        Entry(G.QUAD_SCALE, [block(2), scalar(-1), scalar(1)], [(9, 0)]),
        Entry(G.QUAD_EXTRUDE, [scalar(0), block(4)], [(7, 0)]),
        Entry(G.BOX_TRANSLATE, [scalar(0), block(5), scalar(0)], [(3, 0)]),
        Entry(G.QUAD_DISCARD, [], []),
        Entry(G.QUAD_REPLICATE, [], [(6, 0), (10, 0)]),
        Entry(G.QUAD_GENERATE, [scalar(1)], []),
    ]).to_array()
    rng = np.random.default_rng(seed)
    ax = G.make_axioms(n)
    ax["size"] = rng.uniform(1.0, 3.0, (n, 3)).astype(np.float32)
    ax["position"] = rng.uniform(-5, 5, (n, 3)).astype(np.float32)
    ax["seed"] = np.linspace(0.05, 0.95, n).astype(np.float32)
    ax["block"] = np.arange(n)
    stride = 6
    blocks = np.zeros(n * stride, np.float32)
    for i in range(n):
        blocks[i * stride:(i + 1) * stride] = [rng.uniform(-2, 2), rng.uniform(-2, 2), -rng.uniform(0.5, 1.5),
                                               rng.uniform(0.5, 2.0), rng.uniform(0.2, 1.0), rng.uniform(-1, 1)]
    return {"entries": tab, "axioms": ax, "blocks": blocks, "block_stride": stride, "name": "affine_blocks"}


def test_translate_scale_block_and_size_gradients_match_fp64_central_differences():
    batch = _affine_blocks_batch()
    by_path, gb, gs = _gpu_grad(batch)
    b64 = batch["blocks"].astype(np.float64)
    s64 = batch["axioms"]["size"].astype(np.float64)
    base, keys0 = _loss64(batch, by_path, b64, s64)
    assert base is not None and len(keys0) == len(by_path)

    def block_at(k):
        def f(b, s, h):
            b = b.copy()
            b[k] += h
            return b, s
        return f

    def size_at(k):
        def f(b, s, h):
            s = s.copy()
            s.reshape(-1)[k] += h
            return b, s
        return f

    diffs = [_central(batch, by_path, keys0, base, b64, s64, block_at(k)) for k in range(len(b64))]
    assert _compare("block", gb, diffs) == len(b64)
    # an axiom's Translate/Scale branch reads slots 0..3, its face branch 2, 4, 5
    for i in range(len(batch["axioms"])):
        assert np.count_nonzero(gb[i * 6:(i + 1) * 6]) >= 3, i
    diffs = [_central(batch, by_path, keys0, base, b64, s64, size_at(k)) for k in range(s64.size)]
    assert _compare("size", gs.reshape(-1), diffs) == s64.size


def test_adjoint_requires_tape():
    from operatorgraph_gb300.engine import Engine, PgaError

    b = scenes.menger(0.15)
    eng = Engine(b["entries"])
    out, n, _ = eng.execute(b["axioms"], capacity=1024)
    g = torch.zeros((n, 12), dtype=torch.float32, device="cuda")
    with pytest.raises(PgaError) as e:
        eng.adjoint_raw(g.data_ptr(), None, 0, None)
    assert e.value.status == 8
    eng.release()


def _ref_loss32(batch, by_path, blocks32, sizes32, tmp):
    """sum of W . M over the terminals the REFERENCE's own evaluator derives
    (oracle/_ref, FP32 as the reference computes), matched by the path hash the
    instrumented reference reports; (loss, path set) or (None, None) when a
    terminal's path is unknown."""
    import os

    ax = batch["axioms"].copy()
    ax["size"] = sizes32.reshape(-1, 3)
    entries, ax2 = G.expand_blocks(batch["entries"], ax, blocks32, batch["block_stride"])
    bf, tf = os.path.join(tmp, "b.bin"), os.path.join(tmp, "t.bin")
    G.write_batch_file(bf, entries, ax2)
    oracle.run_reference(bf, tf, entry_mod=len(batch["entries"]))
    t = G.read_terminal_file(tf)
    total, keys = 0.0, []
    for m, p in zip(t["m"].astype(np.float64), t["path"].tolist()):
        w = by_path.get(int(p))
        if w is None:
            return None, None
        total += float(np.dot(w, m))
        keys.append(int(p))
    return total, frozenset(keys)


def test_facade_gradients_match_reference_fp32_central_differences(tmp_path):
    """The adjoint against a gradient taken from the reference's own evaluator:
    central differences of L = sum(W . M) where M are the FP32 transforms the
    reference's SinglePhaseEvaluator derives (oracle/_ref; the batch's
    parameter blocks written into per-axiom table copies), each input moved by
    1% of its size.  4 facades: 64 block parameters and 12 axiom sizes.
    At that step the reference's FP32 differences agree with FP64 differences
    of the restatement to about 6e-5 of the gradient's scale, so the bar is
    the FP64 test's: 2e-3 of the scale."""
    import os

    if not os.path.exists(oracle.REF_HARNESS):
        pytest.skip("oracle/_ref (the reference built from its sources) is not available")
    batch = scenes.facades(4, seed=7)
    by_path, gb, gs = _gpu_grad(batch)
    b32 = batch["blocks"].astype(np.float32)
    s32 = batch["axioms"]["size"].astype(np.float32).reshape(-1)
    tmp = str(tmp_path)
    base, keys0 = _ref_loss32(batch, by_path, b32, s32, tmp)
    assert base is not None and len(keys0) == len(by_path), "the reference's terminals differ from the engine's"

    def diff(vec_b, vec_s, which, k):
        x = (vec_b if which == "b" else vec_s)
        h = np.float32(1e-2 * max(abs(float(x[k])), 0.1))
        out = []
        for sgn in (1, -1):
            bb, ss = vec_b.copy(), vec_s.copy()
            tgt = bb if which == "b" else ss
            tgt[k] = np.float32(tgt[k] + sgn * h)
            step = float(tgt[k]) - float(x[k])  # the step as FP32 represents it
            lv, kv = _ref_loss32(batch, by_path, bb, ss, tmp)
            if lv is None or kv != keys0:
                return None
            out.append((lv, step))
        (lp, hp), (lm, hm) = out
        return (lp - lm) / (hp - hm), (lp - base) / hp, (base - lm) / -hm

    # Facades have no kinks (relative shares only, no Repeat; the side guard
    # sits far from every size), and one-sided FP32 differences carry ~5e-3 of
    # rounding noise, so no kink filter: every central difference is compared.
    tol = RTOL
    for which, got, n in (("b", gb, len(b32)), ("s", gs.reshape(-1), len(s32))):
        diffs = [diff(b32, s32, which, k) for k in range(n)]
        assert all(d is not None for d in diffs), which  # a 1 % step flips no branch here
        scale = max(max(abs(d[0]) for d in diffs), 1.0)
        for k, d in enumerate(diffs):
            assert abs(got[k] - d[0]) <= tol * scale, f"{which}[{k}]: adjoint {got[k]:.6g} vs reference FD {d[0]:.6g}"


def _loss64_vec(batch, paths_sorted, w_sorted, blocks64, sizes64, loss_fn=None):
    """Vectorised FP64 loss over the oracle's double-precision derivation:
    sum(W . M) with W matched by path (paths_sorted / w_sorted sorted by path),
    or loss_fn(M matched to paths_sorted order); (loss, True) or (None, None)
    when the set of paths differs."""
    M, P = oracle.derive_f64(G.DEFAULT_PROCS, batch["entries"], batch["axioms"], blocks64, batch["block_stride"],
                             sizes64)
    if len(P) != len(paths_sorted):
        return None, None
    order = np.argsort(P)
    if not np.array_equal(P[order], paths_sorted):
        return None, None
    Ms = M[order]
    if loss_fn is not None:
        return loss_fn(Ms), True
    return float((Ms * w_sorted).sum()), True


def test_mixed_block_gradients_match_fp64_central_differences():
    """The mixed batch with parameter blocks (scenes.mixed(blocks=True)): the
    buildings' floor heights, tile widths and window wall widths and the
    sponges' split factors, read from per-axiom blocks, get the adjoint's
    gradient; checked with FP64 central differences for every block slot and
    axiom size of 10 axioms (3 sponges, 4 buildings, 3 random grammars)."""
    full = scenes.mixed(64, blocks=True)
    kind = np.where(full["axioms"]["shape"] == G.SHAPE_QUAD, 1, 0)
    quad = np.nonzero(kind == 1)[0][:4]
    box = np.nonzero(kind == 0)[0]
    blk_all = full["blocks"].reshape(-1, scenes.MIXED_STRIDE)
    sponge = [i for i in box if blk_all[i, 0] < 0][:3]
    rand = [i for i in box if blk_all[i, 0] == 0][:3]
    pick = np.array(sorted(list(quad) + sponge + rand))
    ax = full["axioms"][pick].copy()
    ax["block"] = np.arange(len(pick))
    batch = {"entries": full["entries"], "axioms": ax, "blocks": blk_all[pick].reshape(-1).copy(),
             "block_stride": scenes.MIXED_STRIDE}
    by_path, gb, gs = _gpu_grad(batch)
    paths = np.array(sorted(by_path), dtype=np.uint64)
    w = np.array([by_path[int(p)] for p in paths])
    b64 = batch["blocks"].astype(np.float64)
    s64 = batch["axioms"]["size"].astype(np.float64)
    base, _ = _loss64_vec(batch, paths, w, b64, s64)
    assert base is not None

    def fd(vec_b, vec_s, which, k):
        vals = []
        for sgn in (1, -1):
            b, sz = vec_b.copy(), vec_s.copy()
            (b if which == "b" else sz.reshape(-1))[k] += sgn * H
            lv, _ = _loss64_vec(batch, paths, w, b, sz)
            if lv is None:
                return None
            vals.append(lv)
        return (vals[0] - vals[1]) / (2 * H), (vals[0] - base) / H, (base - vals[1]) / H

    diffs = [fd(b64, s64, "b", k) for k in range(len(b64))]
    assert _compare("block", gb, diffs) >= 0.9 * len(b64)
    # every used slot carries gradient: 4 per building, 3 per sponge
    for j, i in enumerate(pick):
        used = 4 if kind[i] == 1 else (3 if blk_all[i, 0] < 0 else 0)
        assert np.count_nonzero(gb[j * 4:j * 4 + used]) == used, (i, gb[j * 4:j * 4 + 4])
    diffs = [fd(b64, s64, "s", k) for k in range(s64.size)]
    assert _compare("size", gs.reshape(-1), diffs) >= 0.8 * s64.size


def test_c4_facade_fitting_through_autograd():
    """Differentiable facade fitting as BASELINE's config 4 states it, on 8
    facades: the target is the terminals of the same trees with every
    parameter moved by N(0, 0.02) (clamped so no branch flips,
    scenes.facade_target_params); the loss is the SSE of terminal centres and
    extents matched by derivation path (autograd.PathTarget); forward and
    adjoint run through torch.autograd.Function.  The gradient matches FP64
    central differences (h = 1e-4) of the same loss on the restatement, and
    40 Adam steps on the parameters cut the loss by more than 10x."""
    from operatorgraph_gb300.autograd import PathTarget, axioms_tensor, derive_transforms
    from operatorgraph_gb300.engine import Engine

    batch = scenes.facades(8, seed=7)
    target_blocks = scenes.facade_target_params(batch["blocks"])
    n_ref = 8 * 384
    eng = Engine(batch["entries"], block_stride=batch["block_stride"], record_tape=True, node_capacity=1 << 18,
                 max_terminals=1 << 16)
    d_ax = axioms_tensor(batch["axioms"])
    sizes = torch.tensor(batch["axioms"]["size"], dtype=torch.float32, device="cuda", requires_grad=True)
    tb = torch.tensor(target_blocks, dtype=torch.float32, device="cuda")
    Mt, pt = derive_transforms(eng, d_ax, tb, sizes.detach(), n_ref)
    target = PathTarget(Mt, pt)
    blocks = torch.tensor(batch["blocks"], dtype=torch.float32, device="cuda", requires_grad=True)
    M, paths = derive_transforms(eng, d_ax, blocks, sizes, n_ref)
    loss = target.sse(M, paths)
    loss.backward()
    g = blocks.grad.detach().cpu().numpy().astype(np.float64)
    # FP64 central differences of the same loss (target values as the GPU derived them)
    tp = target.paths.cpu().numpy().view(np.uint64)  # sorted as signed int64 on the device
    order = np.argsort(tp)
    tp = tp[order]
    tc, te = target.c.cpu().numpy().astype(np.float64)[order], target.e.cpu().numpy().astype(np.float64)[order]

    def sse64(Ms):
        c = Ms[:, [3, 7, 11]]
        R = Ms.reshape(-1, 3, 4)[:, :, :3]
        e = np.sqrt((R * R).sum(axis=1))
        return float(((c - tc) ** 2).sum() + ((e - te) ** 2).sum())

    b64 = batch["blocks"].astype(np.float64)
    s64 = batch["axioms"]["size"].astype(np.float64)
    base, _ = _loss64_vec(batch, tp, None, b64, s64, sse64)
    assert base is not None and abs(base - float(loss.detach())) <= 1e-3 * max(base, 1e-6) + 1e-7
    diffs = []
    for k in range(len(b64)):
        vals = []
        for sgn in (1, -1):
            b = b64.copy()
            b[k] += sgn * H
            lv, _ = _loss64_vec(batch, tp, None, b, s64, sse64)
            vals.append(lv)
        assert None not in vals, k  # the target's perturbation keeps every branch
        diffs.append((vals[0] - vals[1]) / (2 * H))
    # the loss is quadratic, so one-sided differences differ by h f'' and are
    # no kink test here: every central difference is compared
    scale = max(max(abs(d) for d in diffs), 1.0)
    for k, d in enumerate(diffs):
        _check(f"c4[{k}]", g[k], d, scale)
    # fit: Adam on the parameters toward the target
    opt = torch.optim.Adam([blocks], lr=2e-3)
    first = float(loss.detach())
    for _ in range(40):
        opt.zero_grad()
        M, paths = derive_transforms(eng, d_ax, blocks, sizes, n_ref)
        loss = target.sse(M, paths)
        loss.backward()
        opt.step()
    assert float(loss.detach()) < 0.1 * first, (first, float(loss.detach()))
    eng.release()
