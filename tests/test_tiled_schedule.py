"""The page loop of the FP32 tiled stage kernel (csrc/vsl_tiled.cuh), checked on the CPU:
the ring slots the unrolled loop names as compile-time constants are read from the source
and replayed, with the remainder loop's run-time slots, against a model of the ring, for
every block of grids with whole and partial page slabs.

Per page k the kernel reads the centre of page k+3 (the z queue) and the plane of page k
(the x and y stencils), fetches page k+4 and stores it at the end of the page into the
slot of page k-1; one barrier per page separates the pages.  The model checks that every
read finds the page it wants, that no store lands on a slot a later read of the same
page still needs, and that the unrolled slots equal (p - k0) mod RING."""
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(os.path.dirname(HERE), "2018_7_vesicle_gb300", "csrc", "vsl_tiled.cuh")


def schedule():
    src = open(SRC).read()
    ring = int(re.search(r"constexpr int RING = (\d+);", src).group(1))
    calls = re.findall(r"page\(I(\d)\{\}, I(\d)\{\}, I(\d)\{\}, k(?: \+ (\d))?\);", src)
    unrolled = [(int(a), int(b), int(c), int(m or 0)) for a, b, c, m in calls]
    prologue = int(re.search(r"for \(int p = k0; p < k0 \+ (\d+); \+\+p\)", src).group(1))
    ahead = int(re.search(r"fetch\(k \+ (\d+)\);", src).group(1))
    return ring, unrolled, prologue, ahead


def test_unrolled_slots_are_the_ring_positions():
    ring, unrolled, prologue, ahead = schedule()
    assert ring == 5 and len(unrolled) == ring and prologue == ahead == 4
    for sk, sk3, sk4, m in unrolled:
        assert (sk, sk3, sk4) == (m % ring, (m + 3) % ring, (m + ahead) % ring)


def run_block(k0, k1, pges):
    """Replay one block's pages against the ring model; returns the pages computed."""
    ring, unrolled, prologue, ahead = schedule()
    clamp = lambda p: min(max(p, 0), pges - 1)
    slots = [None] * ring
    for p in range(k0, k0 + prologue):  # prologue: pages k0 .. k0+3
        slots[(p - k0) % ring] = clamp(p)
    done = []

    def page(sk, sk3, sk4, k):
        assert slots[sk3] == clamp(k + 3), (k, slots)  # centre of page k+3
        assert slots[sk] == clamp(k), (k, slots)  # plane of page k
        # the slot written at the end must hold a page no later page reads
        old = slots[sk4]
        assert old is None or old <= clamp(k - 1) or old == clamp(k + ahead), (k, old)
        slots[sk4] = clamp(k + ahead)
        done.append(k)

    k = k0
    while k + ring <= k1:  # the unrolled loop
        for sk, sk3, sk4, m in unrolled:
            page(sk, sk3, sk4, k + m)
        k += ring
    r = 0
    while k < k1:  # the remainder with run-time slots
        page(r, (r + 3) % ring, (r + 4) % ring, k)
        k += 1
        r += 1
    return done


def test_every_page_once_for_whole_and_partial_slabs():
    for pges in (1, 3, 4, 5, 7, 16, 20, 23, 96, 256):
        for kz in (1, 2, 3, 4, 5, 6, 8, 10, 16, 20, 25, 32, 40, 64):
            pages = []
            for k0 in range(0, pges, kz):
                pages += run_block(k0, min(k0 + kz, pges), pges)
            assert pages == list(range(pges)), (pges, kz)
