"""World sharding for batched stepping on several GPUs (one process each).

The worlds of a batch are independent spaces, so a job on N GPUs splits
them into N contiguous ranges of world indices with balanced estimated cost,
and each rank steps its range as one batch on its own GPU.  The data path
needs no collective: ranks meet only at a barrier around the timed region,
take the maximum of their step times, and gather per-world results when the
caller asks for them.  The cost of a world is its body count, which sets
its integration, broadphase and (through its contacts) solver work.
"""


def partition(costs, nranks):
    """Contiguous ranges [lo, hi) of indices into `costs`, one per rank,
    with each range's cost sum as close as possible to total / nranks.

    Boundary k is placed at the first index whose prefix sum reaches
    k * total / nranks (or the index before it, whichever is closer), so a
    range never exceeds its share by more than one world's cost.  Ranges
    tile [0, len(costs)) in rank order; a range is empty only when there
    are fewer worlds than ranks."""
    n = len(costs)
    if nranks < 1:
        raise ValueError("nranks must be >= 1")
    if any(c < 0 for c in costs):
        raise ValueError("costs must be non-negative")
    prefix = [0]
    for c in costs:
        prefix.append(prefix[-1] + c)
    total = prefix[-1]
    bounds = [0]
    j = 0
    for k in range(1, nranks):
        target = total * k / nranks
        while j < n and prefix[j + 1] < target:
            j += 1
        # prefix[j] < target <= prefix[j + 1]: cut before or after world j
        cut = j + 1 if (j < n and prefix[j + 1] - target <= target - prefix[j]) else j
        cut = max(cut, bounds[-1])
        # leave at least one world for each remaining rank when possible
        cut = min(cut, n - (nranks - k)) if n >= nranks else min(cut, n)
        cut = max(cut, bounds[-1] + (1 if n >= nranks else 0))
        bounds.append(min(cut, n))
    bounds.append(n)
    return [(bounds[r], bounds[r + 1]) for r in range(nranks)]


def rank_range(costs, rank, nranks):
    """This rank's [lo, hi) range of `partition(costs, nranks)`."""
    return partition(costs, nranks)[rank]
