"""A host model of the mixed trace's warp-scheduled queue (lensMixed.cu, mixedQueue): the same control flow
over 32 lanes a warp, several warps drawing units from one shared counter, rays of random length whose
steps ask for FP64 sub-steps at random.  It checks what the kernel relies on without a GPU: every unit is
traced exactly once, every ray ends after its own number of steps, and every warp's loop ends (no lane
starves), for the default schedule and for the settings at the edges of what the autotuner tries (a round
only when all 32 lanes wait, refills one lane at a time, waits of 1 and 4096 votes)."""
import random

import pytest

INNER_STEPS = 6  # lensMixed.cu kInnerSteps


class Lane:
    def __init__(self):
        self.live = self.exhausted = self.have_step = self.wait_r = self.wait_p = False
        self.unit = -1
        self.k = self.k_end = 0  # this lane's unit: its rays k .. k_end - 1, one after another
        self.left = 0            # steps this ray still takes
        self.taken = 0


def run_queue(units, lengths, p_radial, p_polar, warps=3, batch=32, refill=32, max_wait=256, seed=0, rays=None):
    """units: how many the queue hands out; lengths[u][r]: the steps of ray r of unit u (rays[u] of them; a
    unit of no rays is one outside the frame's band, fetched past).  Returns ({(unit, ray): steps traced},
    loop iterations per warp)."""
    if rays is None:
        lengths = [[n] for n in lengths]
    rng = random.Random(seed)
    counter = [0]
    traced = {}
    state = []
    for _ in range(warps):
        state.append({"lanes": [Lane() for _ in range(32)], "since_start": 0, "since_r": 0, "since_p": 0,
                      "done": False, "iterations": 0, "idle_iterations": 0})
    bound = 50 * (sum(sum(r) for r in lengths) + units) + 1000
    active = list(range(warps))
    while active:
        for w in list(active):
            st, lanes = state[w], state[w]["lanes"]
            st["iterations"] += 1
            assert st["iterations"] < bound, "a warp's loop did not end"
            # the kernel's own argument for its loop's end: every iteration steps some lane's ray, starts
            # rays, runs an FP64 round or ends the loop
            moved = False
            # (1) refill, batched
            idle = [ln for ln in lanes if not ln.live and not ln.exhausted]
            live = [ln for ln in lanes if ln.live]
            if idle and (len(idle) >= refill or not live or st["since_start"] >= max_wait):
                st["since_start"] = 0
                fetch = [ln for ln in idle if ln.unit < 0 or ln.k >= ln.k_end]  # (done with its unit's rays)
                base = counter[0]
                counter[0] += len(fetch)
                for rank, ln in enumerate(fetch):
                    ln.unit = base + rank
                    if ln.unit >= units:
                        ln.exhausted, ln.unit = True, -1
                    else:
                        ln.k, ln.k_end = 0, len(lengths[ln.unit])  # (no rays: fetched again next time)
                for ln in idle:
                    if not ln.live and ln.unit >= 0 and ln.k < ln.k_end:
                        ln.live, ln.left, ln.taken = True, lengths[ln.unit][ln.k], 0
                        moved = True
            elif idle:
                st["since_start"] += 1
            if all(ln.exhausted and not ln.live for ln in lanes):
                active.remove(w)
                continue
            # (2) FP64 rounds: when enough lanes wait, when no lane can move, or after a bounded wait
            ready = [ln for ln in lanes if ln.live and not ln.wait_r and not ln.wait_p]
            need_r = [ln for ln in lanes if ln.wait_r]
            need_p = [ln for ln in lanes if ln.wait_p]
            if need_r and (len(need_r) >= batch or not ready or st["since_r"] >= max_wait):
                for ln in need_r:
                    ln.wait_r = False
                st["since_r"] = 0
                moved = True
            elif need_r:
                st["since_r"] += 1
            if need_p and (len(need_p) >= batch or not ready or st["since_p"] >= max_wait):
                for ln in need_p:
                    ln.wait_p = False
                st["since_p"] = 0
                moved = True
            elif need_p:
                st["since_p"] += 1
            # (3) up to INNER_STEPS FP32 steps a lane between votes
            for _ in range(INNER_STEPS):
                for ln in lanes:
                    if ln.have_step and not ln.wait_r and not ln.wait_p:
                        moved = True
                        ln.have_step = False
                        ln.taken += 1
                        ln.left -= 1
                        if ln.left == 0:
                            assert (ln.unit, ln.k) not in traced, "a ray traced twice"
                            traced[(ln.unit, ln.k)] = ln.taken
                            ln.live = False
                            ln.k += 1
                    if ln.live and not ln.have_step:
                        ln.have_step = True
                        ln.wait_r = rng.random() < p_radial
                        ln.wait_p = rng.random() < p_polar
            # (an iteration that only counts idle lanes towards a refill or a wait is allowed: the counts
            # are bounded, and the wait is over once every live lane waits)
            st["idle_iterations"] = 0 if moved else st["idle_iterations"] + 1
            assert st["idle_iterations"] <= 2, "an iteration with no progress followed another"
    return traced, [s["iterations"] for s in state]


SCHEDULES = [dict(batch=32, refill=32, max_wait=256),   # the defaults
             dict(batch=32, refill=1, max_wait=4096),   # rounds only when all wait or none can move
             dict(batch=1, refill=32, max_wait=1),
             dict(batch=24, refill=8, max_wait=16),
             dict(batch=32, refill=32, max_wait=10 ** 9)]  # (waits that never run out on their own)


@pytest.mark.parametrize("schedule", SCHEDULES)
@pytest.mark.parametrize("need", [(0.0, 0.0), (0.05, 0.04), (0.5, 0.5), (1.0, 1.0)])
def test_every_ray_traced_once_and_every_warp_ends(schedule, need):
    """A ray a unit (the planes of several rays a pixel), and a pixel a unit whose rays one lane traces in
    turn, some units outside the band."""
    rng = random.Random(7)
    units = 400
    one = [[rng.choice([1, 2, rng.randint(3, 60), 192])] for _ in range(units)]
    pixels = [[rng.choice([1, rng.randint(3, 60), 192]) for _ in range(rng.choice([0, 1, 4, 4, 9]))]
              for _ in range(units)]
    for lengths in (one, pixels):
        traced, iterations = run_queue(units, lengths, need[0], need[1], **schedule, seed=3, rays=True)
        want = {(u, r): n for u in range(units) for r, n in enumerate(lengths[u])}
        assert traced == want
        assert all(i > 0 for i in iterations)


def test_no_units_and_fewer_units_than_lanes():
    assert run_queue(0, [], 0.1, 0.1)[0] == {}
    traced, _ = run_queue(5, [3, 1, 192, 7, 2], 0.3, 0.3, warps=4)
    assert traced == {(0, 0): 3, (1, 0): 1, (2, 0): 192, (3, 0): 7, (4, 0): 2}
