"""Batched ensemble over several processes (one GPU each), with members of
failed ranks run again by the others.

A batched ensemble is a set of independent wavepackets, so ranks share no
data while they propagate: members are assigned largest-processing-time
first, every rank runs its members, and each finished member's result goes
to a key-value store (``torch.distributed.TCPStore``, or any object with
``set``, ``get``, ``check``, ``compare_set`` and ``add``).  The store is the
only shared state:

* ``claim/<i>``  the rank running member i (set atomically with compare_set);
* ``done/<i>``   the result of member i (the first one written stays);
* ``hb/<r>``     rank r's heartbeat (wall-clock seconds), written by a
                 background thread every ``timeout / 4`` seconds;
* ``left/<r>``   rank r left after every member was done.

A rank whose heartbeat is older than ``timeout`` and that has not left is
dead: once a rank has run its own members it claims the unfinished members
of dead ranks (compare_set on the claim, so one survivor takes each) and
runs them.  Results are deterministic per member, so a member run twice (a
slow rank taken for dead) gives the same result either way.  The store's
host (rank 0 for a TCPStore) is not covered: it holds the store.
"""
import pickle
import threading
import time


def lpt_partition(costs, nparts):
    """Largest-processing-time-first assignment of independent members to ranks:
    (member lists per rank, in ascending order; loads)."""
    order = sorted(range(len(costs)), key=lambda i: -costs[i])
    loads = [0.0] * nparts
    parts = [[] for _ in range(nparts)]
    for i in order:
        r = min(range(nparts), key=lambda k: loads[k])
        parts[r].append(i)
        loads[r] += costs[i]
    return [sorted(p) for p in parts], loads


class ShardedEnsemble:
    def __init__(self, store, rank, world, costs, timeout=10.0):
        self.store, self.rank, self.world = store, rank, world
        self.n = len(costs)
        self.parts, self.loads = lpt_partition(costs, world)
        self.timeout = float(timeout)
        self._stop = threading.Event()
        self._hb = None

    # ---- store helpers
    def _has(self, key):
        return self.store.check([key])

    def _get(self, key):
        return self.store.get(key)

    def _beat(self):
        self.store.set(f"hb/{self.rank}", repr(time.time()))

    def _heartbeat_loop(self):
        while not self._stop.wait(self.timeout / 4):
            self._beat()

    def _alive(self, r):
        if r == self.rank:
            return True
        if self._has(f"left/{r}"):
            return True
        if not self._has(f"hb/{r}"):
            return True  # not started yet: give it the benefit of the doubt
        return time.time() - float(self._get(f"hb/{r}").decode()) < self.timeout

    def _claim(self, i, expected):
        key = f"claim/{i}"
        got = self.store.compare_set(key, expected, str(self.rank))
        return (got.decode() if isinstance(got, bytes) else got) == str(self.rank)

    def _owner(self, i):
        key = f"claim/{i}"
        return int(self._get(key).decode()) if self._has(key) else None

    def _finish(self, i, result):
        key = f"done/{i}"
        if not self._has(key):
            self.store.set(key, pickle.dumps(result))

    # ---- the run
    def run(self, work, poll=0.05):
        """Run this rank's members with ``work(i) -> result``, then the
        unfinished members of dead ranks; returns the members this rank ran."""
        ran = []
        self._beat()
        self._hb = threading.Thread(target=self._heartbeat_loop, daemon=True)
        self._hb.start()
        try:
            for i in self.parts[self.rank]:
                if self._has(f"done/{i}") or not self._claim(i, ""):
                    continue
                self._finish(i, work(i))
                ran.append(i)
            while True:
                pending = [i for i in range(self.n) if not self._has(f"done/{i}")]
                if not pending:
                    break
                for i in pending:
                    owner = self._owner(i)
                    home = next(r for r in range(self.world) if i in self.parts[r])
                    if owner is None and self._alive(home):
                        continue  # its rank has not reached it yet
                    if owner is not None and self._alive(owner):
                        continue
                    if self._claim(i, "" if owner is None else str(owner)):
                        self._finish(i, work(i))
                        ran.append(i)
                time.sleep(poll)
            # every member is done: leaving now strands nothing
            self.store.set(f"left/{self.rank}", "1")
        finally:
            # a rank that fails stops beating and is taken for dead after timeout
            self._stop.set()
        return ran

    def gather(self):
        """Every member's result, read from the store."""
        return {i: pickle.loads(self._get(f"done/{i}")) for i in range(self.n)}
