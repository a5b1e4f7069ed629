"""The index arithmetic of the bucket-ordered queues, restated on the CPU.

The wavefront shade kernel (wavefront.cu: wf_shade_kernel) and ReSTIR's candidate pass
(restir.cu: queued_pixel) read the material-bucket queues laid end to end, each queue padded
to a multiple of the block so that a block shades one bucket with that bucket's lobe-set
variant; the shade grid gets one block more per bucket (launch_shade), the candidate pass's
grid the same (restir_passes).  For random queue counts, every thread's index must lie inside
its bucket's queue, every queued entry must be read exactly once, and with padding no block may
span two buckets.  Threads in a queue's padding read nothing.
"""
import numpy as np

BLOCK = 128
HIT_BUCKETS = 4


def _padded(n: int) -> int:
    return -(-n // BLOCK) * BLOCK


def _queued_pixel(q: int, counts, pad: bool):
    """restir.cu: queued_pixel<PAD> -> (bucket, index in the bucket's queue) or None."""
    start = 0
    for b in range(HIT_BUCKETS):
        n = counts[b]
        if q < start + n:
            return b, q - start
        start += _padded(n) if pad else n
        if q < start:
            return None
    return None


def _shade_entry(q: int, counts, variants: bool):
    """wavefront.cu: wf_shade_kernel's bucket ranges -> (block bucket, (bucket, index) or None)."""
    start, have, bucket, at = 0, False, HIT_BUCKETS, None
    for k in range(HIT_BUCKETS):
        cnt = counts[k]
        span = _padded(cnt) if variants else cnt
        inside = not have and start <= q < start + cnt
        if bucket == HIT_BUCKETS and start <= q < start + span:
            bucket = k
        if inside:
            at = (k, q - start)
        have = have or inside
        start += span
    return bucket, at


def _random_counts(rng, total: int):
    cuts = np.sort(rng.integers(0, total + 1, HIT_BUCKETS - 1))
    counts = np.diff(np.concatenate([[0], cuts, [rng.integers(cuts[-1], total + 1)]])).tolist()
    if rng.random() < 0.3:
        counts[int(rng.integers(0, HIT_BUCKETS))] = 0
    return counts


def _check(read, grid_blocks: int, counts, padded: bool):
    seen, block_bucket = set(), {}
    for q in range(grid_blocks * BLOCK):
        bucket, entry = read(q)
        if entry is not None:
            b, i = entry
            assert 0 <= i < counts[b], (counts, q, entry)
            assert entry not in seen
            seen.add(entry)
            assert bucket == b
        if padded and bucket < HIT_BUCKETS:
            assert block_bucket.setdefault(q // BLOCK, bucket) == bucket, (counts, q)
    assert len(seen) == sum(counts)


def test_queue_ranges():
    rng = np.random.default_rng(7)
    for _ in range(300):
        total = int(rng.integers(1, 3000))
        counts = _random_counts(rng, total)
        for pad in (False, True):
            grid = -(-total // BLOCK) + (HIT_BUCKETS if pad else 0)

            def read(q, pad=pad):  # a thread without an entry returns before the variant dispatch
                r = _queued_pixel(q, counts, pad)
                return (r[0], r) if r is not None else (HIT_BUCKETS, None)

            _check(read, grid, counts, pad)
            _check(lambda q, v=pad: _shade_entry(q, counts, v), -(-total // BLOCK) + HIT_BUCKETS, counts, pad)


def test_padding_reads_nothing():
    # a thread in the padding after bucket 0 reads nothing (an index past its queue, or one taken
    # from the next queue with the wrong offset, would be an out-of-range read on the device)
    counts = [5, 200, 0, 7]
    assert _queued_pixel(5, counts, True) is None
    assert _queued_pixel(BLOCK - 1, counts, True) is None
    assert _queued_pixel(BLOCK, counts, True) == (1, 0)
    assert _shade_entry(BLOCK - 1, counts, True) == (0, None)
    assert _shade_entry(BLOCK, counts, True) == (1, (1, 0))
