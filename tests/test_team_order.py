"""The team POTRF dataflow's claim order (the device table, computed on the
host by ttg_team_item): every item of the factorisation exactly once, every
wait on a state that an earlier claim produces, and random interleavings of
1..32 blocks always finish with every block final.  CPU only."""
import ctypes
import random

import pytest

import tasktorrent_gb300 as t


def items(P):
    out = []
    k, p, bi, bj = (ctypes.c_int32() for _ in range(4))
    idx = 0
    while True:
        assert t.lib().ttg_team_item(P, idx, ctypes.byref(k), ctypes.byref(p), ctypes.byref(bi), ctypes.byref(bj)) == t.TTG_OK
        if k.value < 0:
            return out
        out.append(("FRT"[k.value], p.value, bi.value, bj.value))
        idx += 1


def deps(it):
    kind, p, bi, bj = it
    if kind == "F":  # panel block (p, p-1), last update and factor of block (p, p)
        return [((p - 1, p - 1), p), ((p, p - 1), p - 1), ((p, p), p - 1)] if p >= 1 else []
    if kind == "R":
        return [((p, p), p + 1), ((bi, p), p)]
    return [((bi, p), p + 1), ((bj, p), p + 1), ((bi, bj), p)]


def outputs(it):
    kind, p, bi, bj = it
    if kind == "F":
        return ([((p, p - 1), p)] if p >= 1 else []) + [((p, p), p + 1)]
    return [((bi, p), p + 1)] if kind == "R" else [((bi, bj), p + 1)]


@pytest.mark.parametrize("P", list(range(1, 45)))
def test_every_item_once_and_waits_on_earlier_claims(P):
    order = items(P)
    want = {("F", j, j, j) for j in range(P)} | {("R", j, i, j) for j in range(P) for i in range(j + 2, P)} | \
        {("T", p, i, q) for p in range(P) for q in range(p + 1, P) for i in range(q, P) if not (i == q == p + 1)}
    assert len(order) == len(set(order)) and set(order) == want
    made = {}
    for k, it in enumerate(order):
        for key in outputs(it):
            made[key] = k
    for k, it in enumerate(order):
        for key, v in deps(it):
            if v > 0:
                assert made[(key, v)] < k, (it, key, v)


@pytest.mark.parametrize("P,K", [(1, 1), (2, 3), (5, 1), (8, 2), (16, 7), (16, 32), (44, 5)])
def test_random_interleavings_finish(P, K):
    order = items(P)
    for seed in range(3):
        rnd = random.Random(seed)
        state, claim, done, blocks = {}, 0, 0, [None] * K
        for _ in range(10 ** 7):
            if done == len(order):
                break
            b = rnd.randrange(K)
            if blocks[b] is None:
                if claim < len(order):
                    blocks[b] = order[claim]
                    claim += 1
                continue
            it = blocks[b]
            if all(state.get(key, 0) >= v for key, v in deps(it)):
                for key, v in outputs(it):
                    assert state.get(key, 0) < v
                    state[key] = v
                blocks[b] = None
                done += 1
        assert done == len(order)
        assert all(state[(i, j)] == j + 1 for i in range(P) for j in range(i + 1))
