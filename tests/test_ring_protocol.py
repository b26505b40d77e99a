"""CPU model of the mbarrier ring protocols of the streamed element applies (csrc/stream_apply.cu)
and of the fused learned-smoother sweep (csrc/ml.cu, k_ml_sweep_tc).

Each agent (producer warp, gather warps, consumer groups / warps) is a generator that yields while it
waits; a seeded scheduler interleaves them and completes in-flight copies at random moments. A barrier
is modelled like an mbarrier: an arrival count plus transaction bytes, a phase counter, and a
parity test that succeeds when the phase of the given parity has completed.

The checks: every chunk is processed exactly once, with its own header, gathered x and matrix stage,
and the run never deadlocks -- for the tag-checked waits the kernels use. With the phase parity alone,
waiters that take turns on a ring can run a full ring ahead and pass a barrier whose earlier use is
still pending; the model shows that failure, which is why the kernels check a per-use tag first.
"""
import random

import pytest


class Bar:
    def __init__(self, count):
        self.count, self.pending, self.tx, self.phase = count, count, 0, 0

    def arrive(self, tx=0):
        self.tx += tx
        self.pending -= 1
        self._check()

    def complete(self, b):
        self.tx -= b
        self._check()

    def _check(self):
        if self.pending == 0 and self.tx == 0:
            self.phase += 1
            self.pending = self.count

    def test(self, parity):
        return (self.phase & 1) != parity


def _schedule(tasks, inflight, rnd):
    stall = 0
    while tasks:
        if inflight and rnd.random() < 0.4:
            b, f = inflight.pop(rnd.randrange(len(inflight)))
            f()
            b.complete(1)
            stall = 0
            continue
        name = rnd.choice(list(tasks))
        try:
            r = next(tasks[name])
            stall = stall + 1 if r == 'w' else 0
        except StopIteration:
            del tasks[name]
            stall = 0
        if stall > 20000 and not inflight:
            return False
    return True


def run_f32(nchunk, seed, tags=True, NST=3, NCX=6, NGRP=2, NGW=2):
    """k_stream_elem_f32: connectivity one chunk ahead of the matrices, gather warps fill x slots,
    consumer groups release the slot after the products and the stage after the outputs."""
    rnd = random.Random(seed)
    full_k = [Bar(1) for _ in range(NST)]
    empty_k = [Bar(1) for _ in range(NST)]
    cx_conn = [Bar(1) for _ in range(NCX)]
    cx_x = [Bar(1) for _ in range(NCX)]
    cx_empty = [Bar(1) for _ in range(NCX)]
    hdr, tag, ktag = [None] * NCX, [-1] * NCX, [-1] * NST
    kdata, xdata = [None] * NST, [None] * NCX
    inflight, log, ticket = [], [], [0]

    def ok_tag(t, u):
        return (not tags) or t == u

    def producer():
        def issue_k(m):
            s = m % NST
            if m >= NST:
                while not empty_k[s].test(((m // NST) & 1) ^ 1):
                    yield 'w'
            ktag[s] = m
            full_k[s].arrive(tx=1)
            inflight.append((full_k[s], lambda s=s, v=hdr[m % NCX]: kdata.__setitem__(s, v)))
        i = 0
        while True:
            j = i % NCX
            if i >= NCX:
                while not cx_empty[j].test(((i // NCX) & 1) ^ 1):
                    yield 'w'
            t = ticket[0]
            ticket[0] += 1
            if t >= nchunk:
                break
            hdr[j], tag[j] = ('c', t), i
            cx_conn[j].arrive(tx=1)
            inflight.append((cx_conn[j], lambda: None))
            if i >= 1:
                yield from issue_k(i - 1)
            i += 1
            yield 's'
        if i >= 1:
            yield from issue_k(i - 1)
        for m in range(i, i + max(NGRP, NGW)):
            j = m % NCX
            if m >= NCX:
                while not cx_empty[j].test(((m // NCX) & 1) ^ 1):
                    yield 'w'
            hdr[j], tag[j] = 'end', m
            cx_conn[j].arrive()

    def gather(gw):
        m = gw
        while True:
            j = m % NCX
            while not (ok_tag(tag[j], m) and cx_conn[j].test((m // NCX) & 1)):
                yield 'w'
            h = hdr[j]
            xdata[j] = h
            yield 's'
            cx_x[j].arrive()
            if h == 'end':
                return
            m += NGW

    def consumer(g):
        m = g
        while True:
            j, s = m % NCX, m % NST
            while not (ok_tag(tag[j], m) and cx_x[j].test((m // NCX) & 1)):
                yield 'w'
            h = hdr[j]
            if h == 'end':
                return
            x = xdata[j]
            while not (ok_tag(ktag[s], m) and full_k[s].test((m // NST) & 1)):
                yield 'w'
            k = kdata[s]
            yield 's'
            cx_empty[j].arrive()
            log.append((m, h, x, k))
            yield 's'
            empty_k[s].arrive()
            m += NGRP

    tasks = {'P': producer(), **{f'G{i}': gather(i) for i in range(NGW)}, **{f'C{i}': consumer(i) for i in range(NGRP)}}
    done = _schedule(tasks, inflight, rnd)
    good = done and sorted(m for m, *_ in log) == list(range(nchunk)) and \
        all(h == x == k == ('c', m) for m, h, x, k in log)
    return good


def run_rowlane(nchunk, seed, tags=True, NST=7, NOWN=4):
    """k_stream_rowlane: one ring of stages, owners take stages in turn."""
    rnd = random.Random(seed)
    full = [Bar(1) for _ in range(NST)]
    empty = [Bar(1) for _ in range(NST)]
    hdr, tag, data = [None] * NST, [-1] * NST, [None] * NST
    inflight, log = [], []

    def producer():
        it = 0
        while True:
            s = it % NST
            if it >= NST:
                while not empty[s].test(((it // NST) & 1) ^ 1):
                    yield 'w'
            if it >= nchunk:
                break
            hdr[s], tag[s] = ('c', it), it
            full[s].arrive(tx=1)
            inflight.append((full[s], lambda s=s, v=('c', it): data.__setitem__(s, v)))
            it += 1
            yield 's'
        for _ in range(NOWN):
            s = it % NST
            if it >= NST:
                while not empty[s].test(((it // NST) & 1) ^ 1):
                    yield 'w'
            hdr[s], tag[s] = 'end', it
            full[s].arrive()
            it += 1

    def owner(w):
        it = w
        while True:
            s = it % NST
            while not ((not tags or tag[s] == it) and full[s].test((it // NST) & 1)):
                yield 'w'
            h = hdr[s]
            if h == 'end':
                return
            log.append((it, h, data[s]))
            yield 's'
            empty[s].arrive()
            it += NOWN

    tasks = {'P': producer(), **{f'W{i}': owner(i) for i in range(NOWN)}}
    done = _schedule(tasks, inflight, rnd)
    return done and sorted(m for m, *_ in log) == list(range(nchunk)) and \
        all(h == d == ('c', m) for m, h, d in log)


def run_mlsweep(ntile, seed, commit_after_mma2=False, free_early=False):
    """k_ml_sweep_tc: 4 gather warps fill feature buffer i & 1 (f_full, count 4) once the MMA that
    read it has completed (f_empty); the compute group issues MMA1 (commit -> f_empty, mma_done), reads
    H, writes G, issues MMA2 (commit -> mma_done) and reads Y. MMAs complete asynchronously.
    `free_early` models a wrong protocol that frees the buffer when MMA1 is issued instead of when it
    completes."""
    rnd = random.Random(seed)
    f_full = [Bar(4) for _ in range(2)]
    f_empty = [Bar(1) for _ in range(2)]
    mma_done = Bar(1)
    feat, norm = [None, None], [None, None]
    tmem, g_buf = [None], [None]
    inflight, log = [], []

    def gather(wid):
        for i in range(ntile):
            b = i & 1
            if i >= 2:
                while not f_empty[b].test(((i >> 1) - 1) & 1):
                    yield 'w'
            if wid == 0:
                feat[b], norm[b] = ('f', i), ('s', i)
            yield 's'
            f_full[b].arrive()

    def compute():
        phase = 0
        for i in range(ntile):
            b = i & 1
            while not f_full[b].test((i >> 1) & 1):
                yield 'w'
            s = norm[b]
            # MMA1 reads the feature buffer when it completes
            src = b
            # both commits track the same MMA: they arrive together once it has read its operands
            mma_done.arrive(tx=1)
            if free_early:
                f_empty[b].arrive()
            else:
                f_empty[b].arrive(tx=1)

            def mma1_done(src=src, b=b):
                tmem[0] = ('H', feat[src])
                if not free_early:
                    f_empty[b].complete(1)
            inflight.append((mma_done, mma1_done))
            while not mma_done.test(phase):
                yield 'w'
            phase ^= 1
            h = tmem[0]
            g_buf[0] = ('G', h)
            yield 's'
            mma_done.arrive(tx=1)
            inflight.append((mma_done, lambda: tmem.__setitem__(0, ('Y', g_buf[0]))))
            while not mma_done.test(phase):
                yield 'w'
            phase ^= 1
            log.append((i, s, tmem[0]))

    tasks = {'C': compute(), **{f'G{w}': gather(w) for w in range(4)}}
    done = _schedule(tasks, inflight, rnd)
    return done and [m for m, *_ in log] == list(range(ntile)) and \
        all(s == ('s', m) and y == ('Y', ('G', ('H', ('f', m)))) for m, s, y in log)


def test_mlsweep_protocol_never_deadlocks_or_mixes_tiles():
    bad = [(n, seed) for n in (1, 2, 3, 4, 7, 20) for seed in range(80) if not run_mlsweep(n, seed)]
    assert not bad, bad[:5]


def test_mlsweep_freeing_at_issue_is_wrong():
    """Freeing the feature buffer when MMA1 is issued (not when it completes) lets the gather of tile
    i + 2 overwrite features that MMA1 of tile i has not read yet."""
    bad = sum(not run_mlsweep(n, seed, free_early=True) for n in (3, 4, 7, 20) for seed in range(80))
    assert bad > 0


SIZES = [1, 2, 3, 5, 7, 13, 40, 150]


@pytest.mark.parametrize("run", [run_f32, run_rowlane])
def test_tagged_rings_never_deadlock_or_mix_chunks(run):
    bad = [(n, seed) for n in SIZES for seed in range(60) if not run(n, seed, tags=True)]
    assert not bad, bad[:5]


@pytest.mark.parametrize("ncx,ngw", [(8, 2), (6, 3), (8, 3)])
def test_f32_slot_and_gather_variants(ncx, ngw):
    """The slot-ring depths and gather-warp counts selectable by stream_f32_variant."""
    bad = [(n, seed) for n in SIZES for seed in range(40) if not run_f32(n, seed, NCX=ncx, NGW=ngw)]
    assert not bad, bad[:5]


@pytest.mark.parametrize("run", [run_f32, run_rowlane])
def test_parity_alone_is_not_enough(run):
    bad = sum(not run(n, seed, tags=False) for n in SIZES for seed in range(60))
    assert bad > 0
