"""The schedule of the device's CSR row compression, checked on the CPU.

`warp_exchange_sort` (simplefem_gb300/csrc/csr_algebra.cu) runs the reference's per-row
exchange sort with merges (sparse/matcsr.cpp:601-622) as a warp-systolic pipeline: lane k
runs pass i + k of each 32-pass sweep one step behind lane k - 1 on a stream of
(column, slot) pairs, the values staying in place and bit 31 of a slot marking a known
zero. `systolic_rows` below replays that schedule lane by lane, step by step, in the
order the kernel's statements run, and the test requires it to keep exactly the entries
of the oracle's serial compression, bit for bit, on rows with repeated columns, exact
cancellations, signed zeros and rows longer than one sweep. The GPU parity tests check
the kernel itself against the same oracle.
"""
import numpy as np
import pytest

ZERO_SLOT = -(1 << 31)   # bit 31 of a slot: the entry is known to be zero
NO_ENTRY = -1


def systolic_rows(c, v):
    """One row through the pipeline: returns the kept (column, value) pairs in order."""
    L = len(c)
    v = list(v)
    cs = [(c[q], q | (ZERO_SLOT if v[q] == 0.0 else 0)) for q in range(L)]
    for i in range(0, L, 32):
        rc, rs = [0] * 32, [0] * 32              # each lane's register (pass i + lane)
        pc, ps = [NO_ENTRY] * 32, [0] * 32       # the entry each lane hands on
        nx = cs[i]
        for s in range((L - i) + 31):
            xc = [nx[0]] + pc[:31]               # shuffle up by one; lane 0 takes the stream
            xs = [nx[1]] + ps[:31]
            nx = cs[i + s + 1] if i + s + 1 < L else (NO_ENTRY, 0)
            npc, nps = [NO_ENTRY] * 32, [0] * 32
            for k in range(32):
                a, sl = xc[k], xs[k]
                valid = a >= 0
                reg = valid and s == 2 * k       # position i + k arrives: it becomes the register
                proc = valid and not reg
                eq = proc and a == rc[k]
                lt = proc and a < rc[k]
                rz, xz = rs[k] < 0, sl < 0
                if eq and not rz and not xz:     # a merge of two nonzeros: the only real add
                    v[rs[k]] = v[rs[k]] + v[sl]
                if eq:
                    if rz:
                        rs[k], sl = sl, rs[k]    # the register takes the other value
                    elif not xz:
                        sl = sl | ZERO_SLOT      # the merged entry is now zero
                oc, os_ = (rc[k], rs[k]) if lt else (a, sl)
                if lt or reg:
                    rc[k], rs[k] = a, sl
                npc[k] = oc if proc else NO_ENTRY
                nps[k] = os_
            pc, ps = npc, nps
            if pc[31] >= 0:                      # lane 31 writes back
                cs[i + s - 31] = (pc[31], ps[31])
            pc[31] = NO_ENTRY
        for k in range(32):
            if i + k < L:
                cs[i + k] = (rc[k], rs[k])
    return [(a, v[sl]) for (a, sl) in cs if sl >= 0 and v[sl] != 0.0]


def _random_rows(seed, count):
    rng = np.random.default_rng(seed)
    rows = []
    for t in range(count):
        L = int(rng.integers(0, 100)) if t % 7 else int(rng.integers(33, 140))
        ncol = int(rng.integers(1, 30))
        c = rng.integers(0, ncol, L).astype(np.int32)
        v = rng.standard_normal(L) * 10.0 ** rng.integers(-6, 7, L)
        if t % 4 == 0:       # explicit zeros of both signs
            z = rng.random(L) < 0.3
            v[z] = np.where(rng.random(int(z.sum())) < 0.5, 0.0, -0.0)
        if t % 5 == 1:       # small integers: exact cancellations
            v = rng.integers(-2, 3, L).astype(np.float64)
        rows.append((c, v))
    return rows


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_systolic_schedule_equals_serial_compression(built, seed):
    from oracle import oracle as O
    O.set_threads(1)
    rows = _random_rows(seed, 120)
    ncols = 30
    A = np.concatenate([[0], np.cumsum([len(c) for c, _ in rows])]).astype(np.int32)
    C = np.concatenate([c for c, _ in rows]).astype(np.int32)
    V = np.concatenate([v for _, v in rows])
    empty = np.zeros(len(rows) + 1, np.int32)
    # the oracle's sum with an empty second operand is its serial compression of each row
    Ao, Co, Vo = O.csr_add(A, C, V, empty, np.zeros(0, np.int32), np.zeros(0), 1.0, 1.0)
    assert int(C.max(initial=0)) < ncols
    for r, (c, v) in enumerate(rows):
        got = systolic_rows(c.tolist(), v.tolist())
        want_c = Co[Ao[r]:Ao[r + 1]]
        want_v = Vo[Ao[r]:Ao[r + 1]]
        assert [g[0] for g in got] == want_c.tolist(), r
        assert np.array_equal(np.array([g[1] for g in got], np.float64).view(np.int64), want_v.view(np.int64)), r
