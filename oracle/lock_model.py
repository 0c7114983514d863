"""Explicit-state models of the path's lock-free protocols, explored over
every interleaving of their atomic steps.  Test infrastructure only: nothing
in the library imports it.

The device code moves its shared words with CAS, atomicMax, atomicAdd and
release stores (include/gpuheap_device.cuh, include/gpuheap_fifo.cuh).  The
hand-offs between blocks, the FIFO ring and the search's termination are
easy to get wrong and cannot be tested exhaustively on a GPU, so they are
modelled here at the level of those atomic steps:

* bottom-up parks (gpuheap_device.cuh `insert_bottomup`, `tryChild`,
  `refill_and_sift`; reference heap/buitdd/heap.cuh:372-418, 636-683):
  an insert that cannot lock its parent parks its node so that deleters
  can pass through it or take it as the last node, then takes it back with
  atomicMax.  Finding its own park value there must prove that nobody held
  the node meanwhile, or the insert would keep a stale copy of the batch.
* the top-down hand-off (`insert_topdown`, `takeLastTopDown`; reference
  heap/tditdd/heap.cuh:371-393, 683-744): a deleter whose last node is an
  insert's target still in flight marks it, and the insert hands its batch
  over at the root instead of writing the target.  The batch must reach
  the deleter exactly once, and neither side may wait forever.
* the FIFO buffer (include/gpuheap_fifo.cuh): pushes publish and pops
  free in reservation and claim order on a ring that wraps, so no key is
  read before it is written or overwritten before it is read.
* termination of a search (gpuheap_gb300/csrc/worklist.cuh): blocks that
  share one heap count themselves busy while they hold work; the search
  must end exactly when the work is done, with no block left waiting.
* the retrieving heap's steal (include/gpuheap_retrieve.cuh; reference
  applications/sssp_longfei_new/heap.cuh:20-35, 147-199, 338-380): a
  retrieve that needs the last node while an insert is still on its way
  down to it takes the insert's batch through the root instead, by the
  per-node word is_taken (0 -> 1 -> 2 -> 3 -> 0).
* the owner-mode delete's lends (gpuheap_gb300/csrc/owner_delete.cuh): a
  level-R node goes to a worker with the carried batch through a reused
  mailbox entry and comes back through its lock word (kLentBack) and a
  reload, while the owner's next plans and passes read its shared copy;
  the taker loads each delete's last node into one of two buffers one
  delete ahead, and a buffer is loaded again only when its reads are over.
* the served device loop's token queue (gpuheap_gb300/csrc/
  search_kernels.cuh, namespace sv): a bounded multi-producer
  multi-consumer ring of per-cell sequence words carries a query's setup
  and search tokens, and the block that retires the last token completes
  the query; requests and completions cross in rings in pinned host memory,
  and the host launches the loop again after an idle exit.
* the bulk delete's ticketed turn at node 0 (gpuheap_device.cuh
  `takeTurn`): blocks take node 0 in the order of their tickets.
* top-down bulk inserts into reserved targets (`insertionReserved`,
  `waitTurn`): they enter the root in target order, or a walk that waits
  at an earlier insert's unwritten target deadlocks against it.
* the retrieving heap's auxiliary buffer (`RetHeapAux::retrieve`), whose
  lock is released while a retrieve reads the heap.
* the FIFO's whole-call push (fifo.cu `k_fifo_bulk_push`): the last block
  to count itself in publishes what the grid copied.

A spin wait is a step that is enabled only when its condition holds, so a
state where no actor can move but some have not finished is a deadlock.
Each model takes switches that plant the mistakes the protocol exists to
prevent; the tests check that the explorer finds them.
"""
from collections import namedtuple
from dataclasses import dataclass, field

# status word values (gpuheap_device.cuh: struct BU, struct TD)
AVAIL, INSHOLD, DELMOD, INUSE = 0, 1, 2, 1 << 30
TD_AVAIL, TD_INUSE, TD_TARGET, TD_MARKED = 0, 1, 2, 3
PARK_BASE = 4  # tickets: PARK_BASE.. (below INUSE)


class Violation(AssertionError):
    """An invariant broke; `trace` is the interleaving that broke it."""

    def __init__(self, msg, trace):
        super().__init__(f"{msg}; trace: {' -> '.join(trace)}")
        self.trace = trace


@dataclass
class Result:
    states: int = 0
    finals: int = 0
    deadlocks: list = field(default_factory=list)
    stuck: list = field(default_factory=list)  # (with progress=True) states that can never finish


def explore(initial, actors, check_final=None, limit=2_000_000, progress=False):
    """Depth-first search over every interleaving.  `initial` is a tuple
    (global state, one program counter per actor); each actor is a function
    (state, pc) -> list of (label, new_state, new_pc), empty when it is
    blocked or done (pc None).  `check_final(state)` runs at every state
    where all actors are done.  Raises Violation from an actor step or the
    final check; returns the number of states and any deadlocks (with the
    trace that reached them).

    With `progress`, the explorer also keeps the state graph and reports in
    `stuck` the states from which no final state can be reached (traces of
    up to three): a livelock, where actors keep moving in a cycle that
    never ends, shows up there though no state is a deadlock."""
    res = Result()
    seen = set()
    succ = {} if progress else None
    parent = {} if progress else None
    finals = []
    stack = [(initial, (), None)]
    while stack:
        (g, pcs), trace, par = stack.pop()
        key = (g, pcs)
        if key in seen:
            if progress and par is not None:
                succ.setdefault(par, set()).add(key)
            continue
        seen.add(key)
        if progress:
            if par is not None:
                succ.setdefault(par, set()).add(key)
            parent[key] = trace
        res.states += 1
        if res.states > limit:
            raise RuntimeError("state space larger than the limit")
        moves = []
        for i, act in enumerate(actors):
            if pcs[i] is None:
                continue
            for label, g2, pc2 in act(g, pcs[i], trace):
                moves.append((i, label, g2, pc2))
        if not moves:
            if all(pc is None for pc in pcs):
                res.finals += 1
                finals.append(key)
                if check_final:
                    check_final(g, list(trace))
            else:
                res.deadlocks.append(list(trace))
            continue
        for i, label, g2, pc2 in moves:
            pcs2 = pcs[:i] + (pc2,) + pcs[i + 1:]
            stack.append(((g2, pcs2), trace + (f"{actors[i].__name__}:{label}",), key))
    if progress:
        pred = {}
        for a, bs in succ.items():
            for b in bs:
                pred.setdefault(b, []).append(a)
        live = set(finals)
        work = list(finals)
        while work:
            b = work.pop()
            for a in pred.get(b, ()):
                if a not in live:
                    live.add(a)
                    work.append(a)
        dead = [k for k in seen if k not in live]
        dead.sort(key=lambda k: len(parent[k]))
        res.stuck = [list(parent[k]) for k in dead[:3]]
    return res


def _set(g, **kw):
    d = g._asdict()
    d.update(kw)
    return type(g)(**d)


# --------------------------------------------------------------------------
# bottom-up parks

BUState = namedtuple("BUState", "x p ver seen_i seen_i2 t_done in_heap")


def bottomup_park_model(tagged=True, trust_own_park=True, delmod_on_release=True, with_taker=True,
                        with_passer=True, park_before_wait=True):
    """Node x with parent p.  Actors:

    * `ins` holds x (INUSE) with its batch cached; p is held by `holder`, so
      its first attempt at p fails and it parks x, locks p, takes x back
      with atomicMax and trusts its cache only if it finds its own park
      value (`insert_bottomup`).
    * `holder` holds p and either releases it, or first passes through x as
      a sifting deleter: atomicMax on x, write x, release x as DELMOD if it
      found a park value (`tryChild`), else as it found it.
    * `taker` takes x as the last node (atomicMax, reset, release AVAIL;
      `refill_and_sift`), after which `ins2` claims x as its new target,
      writes its batch, fails on p and parks x with its own value.

    ver counts writes of x; an insert that trusts its cache asserts that
    ver is what it was at its park.  tagged=False parks every insert with
    the one value INSHOLD (the reference's protocol, which then must never
    trust); delmod_on_release=False restores the raw park value after a
    pass-through; park_before_wait=False makes the insert wait for p while
    it still holds x, against a deleter that holds p and wants x (inserts
    lock child then parent, deleters parent then child: the park is what
    breaks that cycle)."""
    tag_i = PARK_BASE if tagged else INSHOLD
    tag_i2 = PARK_BASE + 1 if tagged else INSHOLD

    def parked(v):
        return v == INSHOLD or PARK_BASE <= v < INUSE

    def ins(g, pc, trace):
        if pc == "try_p":  # one attempt at the parent first
            if g.p == AVAIL:
                return [("cas p ok", _set(g, p=INUSE), "own_p")]
            if not park_before_wait:
                return [("cas p fail; wait holding x", g, "lock_p_holding")]
            return [("cas p fail; park x", _set(g, x=tag_i, seen_i=g.ver), "lock_p")]
        if pc == "lock_p_holding":
            return [("lock p", _set(g, p=INUSE), "own_p")] if g.p == AVAIL else []
        if pc == "lock_p":
            return [("lock p", _set(g, p=INUSE), "retake")] if g.p == AVAIL else []
        if pc == "retake":  # atomicMax(x, INUSE), spinning while INUSE
            if g.x == INUSE:
                return []
            trust = trust_own_park and g.x == tag_i
            if trust and g.ver != g.seen_i:
                raise Violation("insert trusted a stale copy of its parked node", list(trace) + ["ins:retake"])
            return [(f"retake x (found {g.x}, {'trust' if trust else 'reload'})", _set(g, x=INUSE), "own_p")]
        if pc == "own_p":  # write x and p, release both
            return [("write, release x and p", _set(g, x=AVAIL, p=AVAIL, ver=g.ver + 1), None)]
        return []

    def holder(g, pc, trace):
        if pc == "hold":
            moves = [("release p", _set(g, p=AVAIL), None)]
            if with_passer:
                moves.append(("sift toward x", g, "take_x"))
            return moves
        if pc == "take_x":
            if not g.in_heap:  # taken as the last node and not claimed again: the sift finds no child
                return [("x absent, release p", _set(g, p=AVAIL), None)]
            if g.x == INUSE:
                return []
            back = DELMOD if (delmod_on_release and parked(g.x)) else g.x
            return [(f"take x (found {g.x})", _set(g, x=INUSE), ("wrote", back))]
        if isinstance(pc, tuple) and pc[0] == "wrote":
            return [(f"write x, release x as {pc[1]}, release p", _set(g, x=pc[1], ver=g.ver + 1, p=AVAIL), None)]
        return []

    def taker(g, pc, trace):
        if pc == "take":
            if g.x == INUSE:
                return []
            return [(f"take last x (found {g.x})", _set(g, x=INUSE), "reset")]
        if pc == "reset":
            return [("reset x, release AVAIL", _set(g, x=AVAIL, ver=g.ver + 1, t_done=True, in_heap=False), None)]
        return []

    def ins2(g, pc, trace):
        if pc == "claim":  # x is the next target only after the taker lowered the count
            if not g.t_done or g.x != AVAIL:
                return []
            return [("claim x", _set(g, x=INUSE, in_heap=True), "write")]
        if pc == "write":
            return [("write x", _set(g, ver=g.ver + 1), "try_p")]
        if pc == "try_p":
            if g.p == AVAIL:
                return [("cas p ok", _set(g, p=INUSE), "own_p")]
            return [("cas p fail; park x", _set(g, x=tag_i2, seen_i2=g.ver), "lock_p")]
        if pc == "lock_p":
            return [("lock p", _set(g, p=INUSE), "retake")] if g.p == AVAIL else []
        if pc == "retake":
            if g.x == INUSE:
                return []
            trust = trust_own_park and g.x == tag_i2
            if trust and g.ver != g.seen_i2:
                raise Violation("insert trusted a stale copy of its parked node", list(trace) + ["ins2:retake"])
            return [(f"retake x (found {g.x})", _set(g, x=INUSE), "own_p")]
        if pc == "own_p":
            return [("write, release x and p", _set(g, x=AVAIL, p=AVAIL, ver=g.ver + 1), None)]
        return []

    actors = [ins, holder]
    pcs = ["try_p", "hold"]
    if with_taker:
        actors += [taker, ins2]
        pcs += ["take", "claim"]
    g0 = BUState(x=INUSE, p=INUSE, ver=0, seen_i=-1, seen_i2=-1, t_done=not with_taker, in_heap=True)

    def final(g, trace):
        if g.x != AVAIL or g.p != AVAIL:
            raise Violation(f"a lock word left taken (x={g.x}, p={g.p})", trace)

    return (g0, tuple(pcs)), actors, final


# --------------------------------------------------------------------------
# top-down hand-off

TDState = namedtuple("TDState", "t root t_batch got steps")


def topdown_handoff_model(path_steps=2, check_marked_on_path=True, cas_at_target=True, wait_for_handoff=True):
    """One insert on its way down to target t (`path_steps` path nodes still
    ahead) and one deleter that holds the root and wants t as its last node.

    * `ins` checks at every path step whether t was MARKED and then hands
      its batch over at the root; at the end it takes t with
      CAS(TARGET -> INUSE): found MARKED, it hands over; else it writes its
      batch to t and releases it (`insert_topdown`).  A hand-over writes
      the root and turns MARKED back into TARGET.
    * `dele` takes t with CAS(AVAIL -> INUSE), or marks it with
      CAS(TARGET -> MARKED) and then waits for CAS(TARGET -> AVAIL) before
      it reads the root (`takeLastTopDown`).

    got counts the deleter's receipts of the insert's batch: it must be 1
    at the end, from t or from the root, never both.  Planted mistakes:
    the insert ignores MARKED on its path, writes t with a plain store, or
    the deleter reads the root without waiting for the hand-off."""

    def ins(g, pc, trace):
        if isinstance(pc, int):  # pc = path steps still ahead; each reads t first
            if check_marked_on_path and g.t == TD_MARKED:
                return [("sees MARKED on the path", g, "handover")]
            return [(f"path step ({pc} left)", g, pc - 1 if pc > 0 else "at_target")]
        if pc == "at_target":  # a separate step: the deleter may mark t in between
            if cas_at_target:
                if g.t == TD_TARGET:
                    return [("cas t TARGET->INUSE", _set(g, t=TD_INUSE), "write_t")]
                return [(f"cas t fails (found {g.t}): hand over", g, "handover")]
            return [("store t INUSE (no cas)", _set(g, t=TD_INUSE), "write_t")]
        if pc == "write_t":
            return [("write t, release AVAIL", _set(g, t_batch=True, t=TD_AVAIL), None)]
        if pc == "handover":
            return [("write root", _set(g, root=True), "signal")]
        if pc == "signal":
            return [("t MARKED->TARGET", _set(g, t=TD_TARGET), None)]
        return []

    def dele(g, pc, trace):
        if pc == "take":
            moves = []
            if g.t == TD_AVAIL:
                moves.append(("cas t AVAIL->INUSE", _set(g, t=TD_INUSE), "read_t"))
            if g.t == TD_TARGET:
                moves.append(("cas t TARGET->MARKED", _set(g, t=TD_MARKED), "wait"))
            return moves
        if pc == "read_t":
            if not g.t_batch:
                raise Violation("deleter took t before the insert wrote it", list(trace) + ["dele:read_t"])
            return [("read t, reset, release", _set(g, got=g.got + 1, t_batch=False, t=TD_AVAIL), None)]
        if pc == "wait":
            if not wait_for_handoff:
                return [("read root without waiting", g, "read_root")]
            return [("cas t TARGET->AVAIL", _set(g, t=TD_AVAIL), "read_root")] if g.t == TD_TARGET else []
        if pc == "read_root":
            if not g.root:
                raise Violation("deleter read the root before the hand-over", list(trace) + ["dele:read_root"])
            return [("read root", _set(g, got=g.got + 1, root=False), None)]
        return []

    def final(g, trace):
        if g.got != 1 or g.root or g.t_batch:
            raise Violation(f"batch received {g.got} times (root {g.root}, t {g.t_batch})", trace)
        if g.t != TD_AVAIL:
            raise Violation(f"t left in state {g.t}", trace)

    g0 = TDState(t=TD_TARGET, root=False, t_batch=False, got=0, steps=path_steps)
    return (g0, (path_steps, "take")), [ins, dele], final


# --------------------------------------------------------------------------
# termination of a search whose blocks share one heap

TermState = namedtuple("TermState", "heap busy processed")


def termination_model(blocks=2, depth=2, count_while_waiting=False):
    """The busy-counter protocol of gpuheap_gb300/csrc/worklist.cuh
    (`wait_for_keys`, `batch_done`; the reference stops on a count of
    active blocks, applications/sssp_longfei_new/sssp.cu:19-132).

    Work is a binary tree: taking a unit of depth d > 0 inserts two units
    of depth d - 1, one insert at a time; the heap starts with one unit of
    depth `depth`.  Each block loops: wait -> count itself busy -> take a
    unit (or find none) -> insert its children -> uncount -> wait.  A waiting
    block leaves when it reads busy == 0 and then, in a separate step, finds
    the heap empty.  Invariant at the end: every unit was taken, the heap is
    empty and busy is 0; no state may leave blocks waiting on each other.

    count_while_waiting=True plants the mistake the protocol avoids: a
    waiting block counts itself busy, so waiting blocks keep each other
    alive and the search never ends."""
    total = 2 ** (depth + 1) - 1

    def block(g, pc, trace):
        if pc == "wait":
            if count_while_waiting:
                return [("count self while waiting", _set(g, busy=g.busy + 1), "wait_counted")]
            moves = []
            if g.heap:
                moves.append(("sees keys", g, "count"))
            if g.busy == 0:
                moves.append(("reads busy 0", g, "recheck"))
            return moves  # heap empty and others busy: spin
        if pc == "wait_counted":
            moves = []
            if g.heap:
                moves.append(("sees keys", g, "take"))
            if g.busy == 0:
                moves.append(("reads busy 0", g, None))
            return moves
        if pc == "recheck":
            if not g.heap:
                return [("heap empty: leave", g, None)]
            return [("keys again", g, "wait")]
        if pc == "count":
            return [("busy += 1", _set(g, busy=g.busy + 1), "take")]
        if pc == "take":
            if not g.heap:
                return [("empty deleteRoot", g, "done")]
            d = g.heap[0]
            return [(f"take unit {d}", _set(g, heap=g.heap[1:], processed=g.processed + 1), ("ins", d - 1, 2 if d > 0 else 0))]
        if isinstance(pc, tuple) and pc[0] == "ins":
            _, d, left = pc
            if left == 0:
                return [("inserts done", g, "done")]
            return [(f"insert unit {d}", _set(g, heap=tuple(sorted(g.heap + (d,), reverse=True))), ("ins", d, left - 1))]
        if pc == "done":
            return [("busy -= 1", _set(g, busy=g.busy - 1), "wait")]
        return []

    actors = []
    for i in range(blocks):
        def b(g, pc, trace, _f=block):
            return _f(g, pc, trace)
        b.__name__ = f"block{i}"
        actors.append(b)

    def final(g, trace):
        if g.heap or g.busy != 0 or g.processed != total:
            raise Violation(f"search ended with heap {g.heap}, busy {g.busy}, {g.processed}/{total} units", trace)

    return (TermState(heap=(depth,), busy=0, processed=0), tuple(["wait"] * blocks)), actors, final


# --------------------------------------------------------------------------
# the retrieving heap: a retrieve takes the target of an insert in flight

StealState = namedtuple("StealState", "t_lock taken t_batch root got")
T_FREE, T_INS, T_RET = 0, 1, 2


def retrieve_steal_model(path_steps=2, lock_before_check=True, retrieve_locks_target=True, root_before_signal=True):
    """One insert on its way down to its target t (`path_steps` nodes of its
    path still ahead, t the last; it set is_taken[t] = 1 when it started)
    and one retrieve that holds the root's lock and wants t as the last node.

    * `ins` holds the lock of its current node; a step locks the next node
      on the path, releases the current one, then reads is_taken[t]: 2 means
      a retrieve took t, so it releases the node it holds, writes its batch
      into the root (whose lock the retrieve holds) and sets is_taken[t] = 3.
      Reaching t, it writes t, sets is_taken[t] = 0 and releases t.
    * `ret` locks t and reads is_taken[t]: 0, t holds a batch: read it; 1,
      an insert is on its way: set 2, release t, wait for 3, set 0 and read
      the root.

    got counts the retrieve's receipts of the insert's batch: 1 at the end.
    Planted mistakes: the insert reads is_taken before it locks the next
    node, the retrieve reads and sets is_taken without locking t, or the
    insert signals 3 before it has written the root."""

    def ins(g, pc, trace):
        if isinstance(pc, tuple) and pc[0] == "at":  # holds node k's lock
            k = pc[1]
            nxt = k + 1
            if not lock_before_check:
                return [(f"reads is_taken before locking node {nxt}", g, ("late_lock", nxt, g.taken == 2))]
            if nxt == path_steps:  # the target
                if g.t_lock != T_FREE:
                    return []
                return [("locks t, releases its node", _set(g, t_lock=T_INS), ("check", nxt))]
            return [(f"locks node {nxt}, releases node {k}", g, ("check", nxt))]
        if isinstance(pc, tuple) and pc[0] == "late_lock":
            _, nxt, abandon = pc
            if nxt == path_steps:
                if g.t_lock != T_FREE:
                    return []
                g = _set(g, t_lock=T_INS)
            if abandon:
                return [("abandons (read earlier)", _set(g, t_lock=T_FREE) if nxt == path_steps else g, "write_root")]
            return [(f"holds node {nxt}", g, "write_t" if nxt == path_steps else ("at", nxt))]
        if isinstance(pc, tuple) and pc[0] == "check":
            j = pc[1]
            if g.taken == 2:
                return [("sees 2: releases its node", _set(g, t_lock=T_FREE) if j == path_steps else g, "write_root")]
            return [("no steal", g, "write_t" if j == path_steps else ("at", j))]
        if pc == "write_t":
            if g.t_lock != T_INS:
                raise Violation("insert writes t without holding it", list(trace) + ["ins:write_t"])
            return [("writes t, is_taken 0, releases t", _set(g, t_batch=True, taken=0, t_lock=T_FREE), None)]
        if pc == "write_root":
            if root_before_signal:
                return [("writes the root", _set(g, root=True), "signal")]
            return [("sets is_taken 3 first", _set(g, taken=3), "late_root")]
        if pc == "signal":
            return [("is_taken 2 -> 3", _set(g, taken=3), None)]
        if pc == "late_root":
            return [("writes the root", _set(g, root=True), None)]
        return []

    def ret(g, pc, trace):
        if pc == "lock_t":
            if not retrieve_locks_target:
                return [("reads is_taken without the lock", g, "read_taken")]
            if g.t_lock != T_FREE:
                return []
            return [("locks t", _set(g, t_lock=T_RET), "read_taken")]
        if pc == "read_taken":
            if g.taken == 0:
                return [("is_taken 0: t is a node", g, "read_t")]
            if g.taken == 1:
                return [("is_taken 1 -> 2", _set(g, taken=2), "release")]
            raise Violation(f"retrieve found is_taken {g.taken}", list(trace) + ["ret:read_taken"])
        if pc == "read_t":
            if not g.t_batch:
                raise Violation("retrieve read t before the insert wrote it", list(trace) + ["ret:read_t"])
            g = _set(g, got=g.got + 1, t_batch=False)
            return [("reads t, releases t", _set(g, t_lock=T_FREE) if g.t_lock == T_RET else g, None)]
        if pc == "release":
            return [("releases t", _set(g, t_lock=T_FREE) if g.t_lock == T_RET else g, "wait3")]
        if pc == "wait3":
            return [("sees 3, sets 0", _set(g, taken=0), "read_root")] if g.taken == 3 else []
        if pc == "read_root":
            if not g.root:
                raise Violation("retrieve read the root before the insert wrote it", list(trace) + ["ret:read_root"])
            return [("reads the root", _set(g, got=g.got + 1, root=False), None)]
        return []

    def final(g, trace):
        if g.got != 1 or g.root or g.t_batch:
            raise Violation(f"batch received {g.got} times (root {g.root}, t {g.t_batch})", trace)
        if g.taken != 0 or g.t_lock != T_FREE:
            raise Violation(f"t left with is_taken {g.taken}, lock {g.t_lock}", trace)

    g0 = StealState(t_lock=T_FREE, taken=1, t_batch=False, root=False, got=0)
    return (g0, (("at", 0), "lock_t")), [ins, ret], final


# --------------------------------------------------------------------------
# the FIFO buffer

FifoState = namedtuple("FifoState", "slots end write read begin out")


def fifo_model(pushes=(1, 1, 1), pops=(1, 1, 1), capacity=2, wait_room=True, publish_in_order=True,
               claim_by_cas=True, free_in_order=True):
    """gh::Fifo<K> (include/gpuheap_fifo.cuh `push`, `claim`, `copy_out`,
    `release`; reference artifacts/buffer/buffer.cuh:127-213) on a ring of
    `capacity` slots.  Pusher i reserves pushes[i] positions with
    atomicAdd(end), waits until its last slot is within one lap of begin,
    writes its slots one at a time, waits until write reaches its start and
    stores its end.  Popper j takes pops[j] keys in as many pops as it
    needs: it waits until something is published, reads read and write in
    two steps, claims what is there (up to what it still needs) with a CAS
    on read, retrying when it lost, copies its slots one at a time, waits
    until begin reaches its start and stores its end.

    A slot holds (position, key).  Invariants: every copy finds the key
    pushed for that position (each claim is a run of consecutive positions,
    so a popper receives keys in push order), and at the end every key came
    out exactly once and the four positions agree.  Planted mistakes: no room wait, publishing
    without waiting for earlier pushes, claiming with a plain store, and
    freeing without waiting for earlier pops."""
    assert sum(pushes) == sum(pops)
    total = sum(pushes)

    def pusher(i):
        size = pushes[i]

        def push(g, pc, trace):
            if pc == "reserve":
                return [(f"reserve [{g.end},{g.end + size})", _set(g, end=g.end + size), ("room", g.end))]
            kind, start = pc[0], pc[1]
            if kind == "room":
                if wait_room and start + size - g.begin > capacity:
                    return []
                return [("room", g, ("put", start, 0))]
            if kind == "put":
                k = pc[2]
                if k == size:
                    return [("written", g, ("publish", start))]
                pos = start + k
                slots = list(g.slots)
                slots[pos % capacity] = (pos, pos)  # the key pushed for position pos is pos
                return [(f"write slot {pos % capacity} <- {pos}", _set(g, slots=tuple(slots)), ("put", start, k + 1))]
            if kind == "publish":
                if publish_in_order and g.write != start:
                    return []
                return [(f"write = {start + size}", _set(g, write=max(g.write, start + size) if not publish_in_order
                                                         else start + size), None)]
            return []
        push.__name__ = f"push{i}"
        return push

    def popper(j):
        def pop(g, pc, trace):
            # pc[-1] = keys this popper still has to take; it pops until then
            if pc[0] == "wait":
                return [("sees keys", g, ("r", pc[1]))] if g.write > g.read else []
            if pc[0] == "r":
                return [(f"reads read={g.read}", g, ("w", g.read, pc[1]))]
            if pc[0] == "w":
                _, r, left = pc
                n = min(max(g.write - r, 0), left)
                if n == 0:
                    return [("nothing left at r: retry", g, ("wait", left))]
                return [(f"reads write={g.write}", g, ("cas", r, n, left))]
            if pc[0] == "cas":
                _, r, n, left = pc
                if claim_by_cas and g.read != r:
                    return [("cas lost", g, ("wait", left))]
                return [(f"claims [{r},{r + n})", _set(g, read=r + n if claim_by_cas else max(g.read, r + n)),
                         ("copy", r, n, 0, left))]
            if pc[0] == "copy":
                _, start, n, k, left = pc
                if k == n:
                    return [("copied", g, ("free", start, n, left))]
                pos = start + k
                slot = g.slots[pos % capacity]
                if slot != (pos, pos):
                    raise Violation(f"popper read slot {pos % capacity} for position {pos} and found {slot}",
                                    list(trace) + [f"pop{j}:copy {pos}"])
                return [(f"copies {pos}", _set(g, out=g.out + (pos,)), ("copy", start, n, k + 1, left))]
            if pc[0] == "free":
                _, start, n, left = pc
                if free_in_order and g.begin != start:
                    return []
                nxt = ("wait", left - n) if left > n else None
                return [(f"begin = {start + n}", _set(g, begin=start + n if free_in_order else max(g.begin, start + n)),
                         nxt)]
            return []
        pop.__name__ = f"pop{j}"
        return pop

    actors = [pusher(i) for i in range(len(pushes))] + [popper(j) for j in range(len(pops))]
    pcs = tuple(["reserve"] * len(pushes) + [("wait", m) for m in pops])

    def final(g, trace):
        if sorted(g.out) != list(range(total)):
            raise Violation(f"keys out {g.out}, pushed 0..{total - 1}", trace)
        if g.begin != total or g.write != total or g.read != total:
            raise Violation(f"positions end at read {g.read}, write {g.write}, begin {g.begin}", trace)

    g0 = FifoState(slots=tuple([(-1, -1)] * capacity), end=0, write=0, read=0, begin=0, out=())
    return (g0, pcs), actors, final


# --------------------------------------------------------------------------
# the owner-mode delete's lend and return of level-R nodes

LendState = namedtuple("LendState", "node_ver slot_ver lent status req seq data cons reading got")
L_HELD, L_BACK = "L", "B"


def _put(t, i, v):
    return t[:i] + (v,) + t[i + 1:]


def owner_lend_model(deletes=3, nodes=2, mark_after_pass=True, back_after_write=True, returner_checks_status=True,
                     cons_after_load=True, lender_waits_cons=True):
    """The lend round trip of gpuheap_gb300/csrc/owner_delete.cuh: delete d
    lends level-R node d % `nodes` (with nodes = 1 every path runs through
    the same node, the common case; with 2 a lend can go out while the
    previous node is still away), through one mailbox entry that
    consecutive lends reuse.

    * `owner` (the compute warps), per delete d with x = d % nodes: the plan
      waits until lentState[x] is 0 and reads x's shared slot; it posts lend
      d (x and the carried batch); the pass reads the slot (two steps); only
      then lentState[x] = 1.
    * `lender`: copies lend q's carried batch into the mailbox entry once
      the worker has read lend q - 1 from it (cons), then publishes seq.
    * `worker`: takes lend q when seq says so and starts the carried batch's
      bulk load; when the load is in it releases cons (CarriedInFlight),
      writes x's new content to global memory and leaves x's lock word at
      kLentBack.
    * `returner`: for a node with lentState 1 and lock word kLentBack, sets
      the word back to held, reloads the slot from global memory (the bulk
      copy takes the node's version at that moment), then lentState = 0.

    Invariants: a plan reads its node's current version; no reload lands
    while the pass reads that slot; the worker's carried batch is its own
    lend's; at the end every version matches, every node is held and every
    lend was received once.  Planted mistakes: lentState set before the
    pass, kLentBack before the write, a returner that does not look at the
    lock word, cons released when the load starts, a lender that does not
    wait for cons."""

    def owner(g, pc, trace):
        step, d = pc
        x = d % nodes
        if step == "plan":
            if g.lent[x] != 0:
                return []
            if g.slot_ver[x] != g.node_ver[x]:
                raise Violation(f"plan {d} read node {x}'s slot at version {g.slot_ver[x]}, the node is at "
                                f"{g.node_ver[x]}", list(trace) + [f"owner:plan {d}"])
            return [(f"plan {d}", g, ("post", d))]
        if step == "post":
            nxt = ("pass_start", d) if mark_after_pass else ("early_mark", d)
            return [(f"post lend {d} (node {x})", _set(g, req=d + 1), nxt)]
        if step == "early_mark":
            return [(f"lentState[{x}] 1 before the pass", _set(g, lent=_put(g.lent, x, 1)), ("pass_start", d))]
        if step == "pass_start":
            return [(f"pass {d} reads node {x}'s slot", _set(g, reading=x), ("pass_end", d))]
        if step == "pass_end":
            nxt = ("mark", d) if mark_after_pass else ("next", d)
            return [(f"pass {d} done", _set(g, reading=-1), nxt)]
        if step == "mark":
            return [(f"lentState[{x}] 1", _set(g, lent=_put(g.lent, x, 1)), ("next", d))]
        if step == "next":
            return [("next delete", g, ("plan", d + 1) if d + 1 < deletes else None)]
        return []

    def lender(g, pc, trace):
        q = pc
        if g.req <= q:
            return []
        if lender_waits_cons and g.cons != q:
            return []
        return [(f"copies lend {q} into the entry, seq {q + 1}", _set(g, data=q, seq=q + 1),
                 q + 1 if q + 1 < deletes else None)]

    def worker(g, pc, trace):
        step, q = pc
        x = q % nodes
        nxt_lend = ("take", q + 1) if q + 1 < deletes else None
        if step == "take":
            if g.seq != q + 1:
                return []
            g2 = g if cons_after_load else _set(g, cons=q + 1)
            return [(f"takes lend {q}, starts the carried load", g2, ("load_end", q))]
        if step == "load_end":
            if g.data != q:
                raise Violation(f"worker's carried batch for lend {q} is lend {g.data}'s",
                                list(trace) + [f"worker:load_end {q}"])
            g2 = _set(g, cons=q + 1) if cons_after_load else g
            return [(f"carried batch {q} in", _set(g2, got=g.got + 1), ("write", q))]
        if step == "write":
            if back_after_write:
                return [(f"writes node {x}", _set(g, node_ver=_put(g.node_ver, x, g.node_ver[x] + 1)), ("back", q))]
            return [(f"node {x} kLentBack before the write", _set(g, status=_put(g.status, x, L_BACK)),
                     ("late_write", q))]
        if step == "late_write":
            return [(f"writes node {x}", _set(g, node_ver=_put(g.node_ver, x, g.node_ver[x] + 1)), nxt_lend)]
        if step == "back":
            return [(f"node {x} kLentBack", _set(g, status=_put(g.status, x, L_BACK)), nxt_lend)]
        return []

    def returner(g, pc, trace):
        k = pc  # reloads done
        moves = []
        for x in range(nodes):
            if g.lent[x] != 1 or (returner_checks_status and g.status[x] != L_BACK):
                continue
            if g.reading == x:
                raise Violation(f"reload of node {x} lands while the pass reads its slot",
                                list(trace) + [f"returner:reload {x}"])
            g2 = _set(g, status=_put(g.status, x, L_HELD), slot_ver=_put(g.slot_ver, x, g.node_ver[x]),
                      lent=_put(g.lent, x, 0))
            moves.append((f"takes node {x} back at version {g.node_ver[x]}", g2, k + 1 if k + 1 < deletes else None))
        return moves

    def final(g, trace):
        if g.got != deletes:
            raise Violation(f"worker received {g.got} carried batches of {deletes}", trace)
        per = [deletes // nodes + (1 if x < deletes % nodes else 0) for x in range(nodes)]
        if list(g.node_ver) != per or list(g.slot_ver) != per or any(g.lent) or \
                any(st != L_HELD for st in g.status):
            raise Violation(f"end: nodes at {g.node_ver}, slots at {g.slot_ver}, lentState {g.lent}, "
                            f"lock words {g.status}", trace)

    z = (0,) * nodes
    g0 = LendState(node_ver=z, slot_ver=z, lent=z, status=(L_HELD,) * nodes, req=0, seq=0, data=-1, cons=0,
                   reading=-1, got=0)
    return (g0, (("plan", 0), 0, ("take", 0), 0)), [owner, lender, worker, returner], final


# --------------------------------------------------------------------------
# the owner-mode delete's two carried-batch buffers

TakerState = namedtuple("TakerState", "buf ready free allowed computing copying req done_lends")


def owner_taker_model(deletes=4, lends=(True, False, True, True), taker_waits_free=True, free_after_copy=True,
                      compute_waits_ready=True):
    """The carried-batch buffers of gpuheap_gb300/csrc/owner_delete.cuh: the
    taker warp takes delete t's last node into buffer t & 1 one delete
    ahead; delete d's compute warps read buffer d & 1 (refill, plan, general
    steps) and, when d lends its level-R node, the lender warp copies the
    buffer into the mailbox afterwards.

    * `taker`, per t: waits until takeAllowed > t and cFree[b] >= t >> 1
      (both earlier uses of the buffer are over), loads the node into the
      buffer, cReady[b] = t + 1.
    * `compute`, per d: waits for cReady[b] == d + 1, sets takeAllowed =
      d + 2, reads the buffer (two steps); a lending delete posts the
      request for the lender (whose copy then frees the buffer), any other
      frees it itself (cFree[b] += 1).
    * `lender`: copies the buffer of each posted lend (two steps), then
      cFree[b] += 1.

    Invariants: every read finds its own delete's last node and no load
    lands in a buffer that is being read.  Planted mistakes: a taker that
    does not wait for cFree, a lending delete that frees the buffer itself
    (before the lender's copy), compute warps that do not wait for cReady."""
    assert len(lends) == deletes

    def taker(g, pc, trace):
        t = pc
        b = t & 1
        if g.allowed <= t:
            return []
        if taker_waits_free and g.free[b] < (t >> 1):
            return []
        if g.computing == b or g.copying == b:
            raise Violation(f"take {t} loads buffer {b} while it is read", list(trace) + [f"taker:load {t}"])
        g2 = _set(g, buf=_put(g.buf, b, t), ready=_put(g.ready, b, t + 1))
        return [(f"loads delete {t}'s last node into buffer {b}", g2, t + 1 if t + 1 < deletes else None)]

    def compute(g, pc, trace):
        step, d = pc
        b = d & 1
        if step == "wait":
            if compute_waits_ready and g.ready[b] != d + 1:
                return []
            return [(f"delete {d}: buffer {b} ready", _set(g, allowed=max(g.allowed, d + 2)), ("read", d))]
        if step == "read":
            if g.buf[b] != d:
                raise Violation(f"delete {d} reads buffer {b} holding delete {g.buf[b]}'s node",
                                list(trace) + [f"compute:read {d}"])
            return [(f"delete {d} reads buffer {b}", _set(g, computing=b), ("done", d))]
        if step == "done":
            g2 = _set(g, computing=-1)
            nxt = ("wait", d + 1) if d + 1 < deletes else None
            if lends[d]:
                g2 = _set(g2, req=g2.req + (d,))
                if not free_after_copy:
                    g2 = _set(g2, free=_put(g2.free, b, g2.free[b] + 1))
                return [(f"delete {d} posts its lend", g2, nxt)]
            return [(f"delete {d} frees buffer {b}", _set(g2, free=_put(g2.free, b, g2.free[b] + 1)), nxt)]
        return []

    def lender(g, pc, trace):
        step, k = pc  # k = lends copied
        total = sum(lends)
        if step == "wait":
            if len(g.req) <= k:
                return []
            d = g.req[k]
            b = d & 1
            if g.buf[b] != d:
                raise Violation(f"lend of delete {d} copies buffer {b} holding delete {g.buf[b]}'s node",
                                list(trace) + [f"lender:copy {d}"])
            return [(f"copies delete {d}'s buffer {b}", _set(g, copying=b), ("free", k))]
        if step == "free":
            d = g.req[k]
            b = d & 1
            g2 = _set(g, copying=-1, done_lends=g.done_lends + 1)
            if free_after_copy:
                g2 = _set(g2, free=_put(g2.free, b, g2.free[b] + 1))
            return [(f"copied, frees buffer {b}", g2, ("wait", k + 1) if k + 1 < total else None)]
        return []

    def final(g, trace):
        if g.done_lends != sum(lends):
            raise Violation(f"{g.done_lends} lends copied of {sum(lends)}", trace)

    g0 = TakerState(buf=(-1, -1), ready=(0, 0), free=(0, 0), allowed=1, computing=-1, copying=-1, req=(),
                    done_lends=0)
    actors = [taker, compute] + ([lender] if any(lends) else [])
    pcs = (0, ("wait", 0)) + ((("wait", 0),) if any(lends) else ())
    return (g0, pcs), actors, final


# --------------------------------------------------------------------------
# the served device loop's token queue and a query's retirement

TokenState = namedtuple("TokenState", "cells enq deq tokens over stints completed setups")
SETUP, SEARCH = "setup", "search"


def serve_token_model(blocks=2, query_blocks=2, cells=2, max_stints=3, pop_by_cas=True, push_waits_cell=True,
                      release_after_read=True, retire_atomic=True, poll_is_wait=True):
    """The served loop's token queue and retirement (search_kernels.cuh,
    namespace sv: `push`, `pop`, `setup_query`, `end_stint`): a bounded
    multi-producer multi-consumer ring in which cell c serves positions
    c, c + cells, ...; its sequence word is pos when free for position pos,
    pos + 1 when holding pos's token.

    * push: pos = atomicAdd(enq); wait until seq == pos; write the token;
      seq = pos + 1 (release).
    * pop: read deq, then the cell's seq; seq == pos + 1: CAS deq pos ->
      pos + 1, on success read the token and free the cell for pos + cells
      (seq = pos + cells); seq < pos + 1: empty.
    * One query: the admission queued its setup token; the block that pops
      it pushes `query_blocks` search tokens.  A block with a search token
      works a stint; if the search is not over (it may end at any stint,
      and does after `max_stints`) the token goes back, else the block
      decrements the query's token count and the one that takes it to 0
      completes the query.

    A block polling an empty ring is a wait (the loop's stall limit would
    end it), so a query whose tokens are all gone without a completion
    shows up as a deadlock; with `poll_is_wait=False` the poll spins as the
    device code does, and the same fault is a livelock that only the
    explorer's progress check finds.  Invariants: a pop reads the token pushed for
    its position; the query completes exactly once, after every token has
    retired; the ring ends empty.  Planted mistakes: claiming by a plain store instead of a CAS, a
    push that does not wait for its cell, a cell freed before its token is
    read, and a retirement by load and store instead of atomicSub."""

    def put(g, pos, val):
        cs = list(g.cells)
        cs[pos % cells] = (pos + 1, (pos, val))
        return _set(g, cells=tuple(cs))

    def block(i):
        def act(g, pc, trace):
            kind = pc[0]
            if kind == "next":
                if g.completed:
                    return [("leaves", g, None)]
                if g.deq >= g.enq and poll_is_wait:
                    return []  # nothing queued: polls until a token comes (or the loop's stall limit)
                return [(f"reads deq {g.deq}", g, ("seq", g.deq))]
            if kind == "seq":
                pos = pc[1]
                s, _ = g.cells[pos % cells]
                if s == pos + 1:
                    return [(f"cell {pos % cells} holds {pos}", g, ("cas", pos))]
                return [("empty", g, ("next",))]
            if kind == "cas":
                pos = pc[1]
                if pop_by_cas and g.deq != pos:
                    return [("cas lost", g, ("next",))]
                g2 = _set(g, deq=pos + 1 if pop_by_cas else max(g.deq, pos + 1))
                if release_after_read:
                    return [(f"claims {pos}", g2, ("read", pos))]
                cs = list(g2.cells)
                cs[pos % cells] = (pos + cells, cs[pos % cells][1])
                return [(f"claims {pos}, frees its cell first", _set(g2, cells=tuple(cs)), ("read", pos))]
            if kind == "read":
                pos = pc[1]
                _, (wpos, val) = g.cells[pos % cells]
                if wpos != pos:
                    raise Violation(f"block {i} popped position {pos} and read position {wpos}'s token",
                                    list(trace) + [f"b{i}:read {pos}"])
                g2 = g
                if release_after_read:
                    cs = list(g.cells)
                    cs[pos % cells] = (pos + cells, (wpos, val))
                    g2 = _set(g, cells=tuple(cs))
                return [(f"takes {val}", g2, ("got", val))]
            if kind == "got":
                val = pc[1]
                if val == SETUP:
                    if g.setups:
                        raise Violation("the setup token ran twice", list(trace) + [f"b{i}:setup"])
                    return [("sets the query up", _set(g, setups=1), ("push", SEARCH, query_blocks))]
                # a stint; the search may end here
                moves = []
                if not g.over and g.stints < max_stints:
                    moves.append(("stint, search goes on", _set(g, stints=g.stints + 1), ("push", SEARCH, 1)))
                moves.append(("stint, search over", _set(g, over=True, stints=g.stints + 1), ("retire",)))
                if g.over:
                    moves = [("stint, search over", g, ("retire",))]
                return moves
            if kind == "push":
                _, val, left = pc
                if left == 0:
                    return [("pushed", g, ("next",))]
                pos = g.enq
                return [(f"reserves {pos}", _set(g, enq=pos + 1), ("wait", val, left, pos))]
            if kind == "wait":
                _, val, left, pos = pc
                s, _ = g.cells[pos % cells]
                if push_waits_cell and s != pos:
                    return []
                return [(f"writes {val} at {pos}", put(g, pos, val), ("push", val, left - 1))]
            if kind == "retire":
                if retire_atomic:
                    left = g.tokens - 1
                    g2 = _set(g, tokens=left)
                    if left == 0:
                        return [("last token: completes", _set(g2, completed=g2.completed + 1), ("next",))]
                    return [(f"token retires ({left} left)", g2, ("next",))]
                return [(f"reads tokens {g.tokens}", g, ("retire_w", g.tokens))]
            if kind == "retire_w":
                left = pc[1] - 1
                g2 = _set(g, tokens=left)
                if left == 0:
                    return [("writes 0: completes", _set(g2, completed=g2.completed + 1), ("next",))]
                return [(f"writes {left}", g2, ("next",))]
            return []
        act.__name__ = f"b{i}"
        return act

    def final(g, trace):
        if g.completed != 1 or g.tokens != 0:
            raise Violation(f"query completed {g.completed} times, {g.tokens} tokens out", trace)
        if g.deq != g.enq:
            raise Violation(f"ring ends with deq {g.deq}, enq {g.enq}", trace)

    c0 = [(k, (-1, None)) for k in range(cells)]
    c0[0] = (1, (0, SETUP))  # the admission's setup token at position 0
    g0 = TokenState(cells=tuple(c0), enq=1, deq=0, tokens=query_blocks, over=False, stints=0, completed=0,
                    setups=0)
    return (g0, tuple(("next",) for _ in range(blocks))), [block(i) for i in range(blocks)], final


# --------------------------------------------------------------------------
# the served device loop's request and completion rings (pinned host memory)

RingState = namedtuple("RingState", "req posted taken admitted claim done consumed claimed")


def serve_rings_model(queries=4, cap=2, completers=2, guard_by_completions=True, seq_after_fields=True,
                      take_after_copy=True):
    """The host <-> device rings of the served loop (gpuheap_gb300/csrc/
    serve.cu `post_requests`, `gh_serve_poll`; search_kernels.cuh `admit`,
    `complete`).  Both rings have `cap` records; record k of a ring holds
    item k when its seq word is k + 1.

    * `host`: posts request p into record p % cap (fields, then seq with a
      release store) while p - consumed < cap, consumed counting the
      completions it has read; reads completion c when its seq is c + 1.
    * `admit` (device, lock held): copies request `taken` when its seq says
      so, then publishes taken + 1; the query is then active.
    * `complete` x `completers` (device blocks): any active query may end
      next; its block claims completion number c (lock held), writes the
      record's fields, then its seq.

    Invariants: the device copies the request posted for that number; the
    host reads completion c as the query claimed with c; no completion
    record is written while the host has yet to read the one it replaces;
    every query completes.  Planted mistakes: posting while p - taken < cap
    (counting admissions instead of completions) and a completion's seq
    written before its fields.  `take_after_copy=False` publishes taken
    before the copy: still safe, because the host reuses a request record
    only after that request's completion (taken is only reported)."""

    def host(g, pc, trace):
        moves = []
        step = pc[0]
        if step == "idle":
            limit = g.consumed if guard_by_completions else g.taken
            if g.posted < queries and g.posted - limit < cap:
                p = g.posted
                req = list(g.req)
                req[p % cap] = (req[p % cap][0], p)  # fields
                moves.append((f"writes request {p}", _set(g, req=tuple(req)), ("publish", p)))
            c = g.consumed
            if c < queries and g.done[c % cap][0] == c + 1:
                qid = g.done[c % cap][1]
                if qid != g.claimed[c]:
                    raise Violation(f"host read completion {c} as query {qid}, claimed by query {g.claimed[c]}",
                                    list(trace) + [f"host:read {c}"])
                nxt = "idle" if c + 1 < queries else None
                moves.append((f"reads completion {c} (query {qid})", _set(g, consumed=c + 1), (nxt,) if nxt else None))
            return moves
        if step == "publish":
            p = pc[1]
            req = list(g.req)
            req[p % cap] = (p + 1, req[p % cap][1])
            return [(f"publishes request {p}", _set(g, req=tuple(req), posted=p + 1), ("idle",))]
        return []

    def admit(g, pc, trace):
        t = g.taken
        if t >= queries or g.req[t % cap][0] != t + 1:
            return []
        if take_after_copy:
            content = g.req[t % cap][1]
            if content != t:
                raise Violation(f"device copied request {t} and found request {content}'s fields",
                                list(trace) + [f"admit:copy {t}"])
            return [(f"copies request {t}, taken {t + 1}", _set(g, taken=t + 1, admitted=g.admitted + (t,)),
                     "idle" if t + 1 < queries else None)]
        return [(f"taken {t + 1} before the copy", _set(g, taken=t + 1), ("late_copy", t))]

    def admit_wrap(g, pc, trace):
        if pc == "idle":
            return admit(g, pc, trace)
        if isinstance(pc, tuple) and pc[0] == "late_copy":
            t = pc[1]
            content = g.req[t % cap][1]
            if content != t:
                raise Violation(f"device copied request {t} and found request {content}'s fields",
                                list(trace) + [f"admit:late copy {t}"])
            return [(f"copies request {t}", _set(g, admitted=g.admitted + (t,)),
                     "idle" if t + 1 < queries else None)]
        return []
    admit_wrap.__name__ = "admit"

    def completer(k):
        def act(g, pc, trace):
            if pc == "idle":
                moves = []
                for q in g.admitted:
                    c = g.claim
                    claimed = g.claimed[:c] + (q,) + g.claimed[c + 1:]
                    left = tuple(x for x in g.admitted if x != q)
                    moves.append((f"query {q} ends, claims completion {c}",
                                  _set(g, admitted=left, claim=c + 1, claimed=claimed), ("write", c, q)))
                if g.claim >= queries:
                    return [("leaves", g, None)]
                return moves
            step, c, q = pc
            slot = c % cap
            if step == "write":
                old_seq = g.done[slot][0]
                if old_seq != 0 and old_seq - 1 >= g.consumed:
                    raise Violation(f"completion {c} overwrites completion {old_seq - 1} before the host read it",
                                    list(trace) + [f"c{k}:write {c}"])
                done = list(g.done)
                if seq_after_fields:
                    done[slot] = (old_seq, q)
                    return [(f"writes completion {c}'s fields", _set(g, done=tuple(done)), ("seq", c, q))]
                done[slot] = (c + 1, done[slot][1])
                return [(f"completion {c}: seq first", _set(g, done=tuple(done)), ("late_fields", c, q))]
            if step == "seq":
                done = list(g.done)
                done[slot] = (c + 1, done[slot][1])
                return [(f"publishes completion {c}", _set(g, done=tuple(done)), "idle")]
            if step == "late_fields":
                done = list(g.done)
                done[slot] = (done[slot][0], q)
                return [(f"writes completion {c}'s fields", _set(g, done=tuple(done)), "idle")]
            return []
        act.__name__ = f"c{k}"
        return act

    def final(g, trace):
        if g.consumed != queries or g.admitted:
            raise Violation(f"host read {g.consumed} of {queries} completions, {len(g.admitted)} still active", trace)

    g0 = RingState(req=tuple((0, -1) for _ in range(cap)), posted=0, taken=0, admitted=(), claim=0,
                   done=tuple((0, -1) for _ in range(cap)), consumed=0, claimed=(-1,) * queries)
    actors = [host, admit_wrap] + [completer(k) for k in range(completers)]
    return (g0, (("idle",), "idle") + ("idle",) * completers), actors, final


# --------------------------------------------------------------------------
# the served device loop's launch, idle exit and relaunch

LoopState = namedtuple("LoopState", "posted taken active completed consumed running armed")


def serve_loop_model(requests=2, relaunch_on_poll=True):
    """The served loop's lifetime (gpuheap_gb300/csrc/serve.cu
    `gh_serve_poll`, `launch_loop`; search_kernels.cuh `admit`): the device
    loop leaves after an idle limit with nothing pending or active, and the
    host launches it again from its poll whenever requests it posted have
    not all completed.

    * `host`: posts `requests` requests one by one; a poll reads every
      completion there is, stops once all are read, and otherwise, if the
      loop's launch has ended, launches it again.
    * `device` (the admitting block, while launched): takes a posted
      request (it becomes active), or completes an active one, or, seeing
      nothing pending or active, arms the idle limit; with the limit armed
      and the ring still empty when it looks, it decides to leave, and
      leaves in a later step (the host may post in between).

    Explored with progress=True: from every state every request can still
    complete.  Planted mistake: a host that launches the loop only when it
    posts, so that a request posted between the loop's last look at the
    ring and its exit is stranded."""

    def host(g, pc, trace):
        moves = []
        if pc == "run":
            if g.posted < requests:
                g2 = _set(g, posted=g.posted + 1)
                if not relaunch_on_poll and not g.running:
                    g2 = _set(g2, running=True, armed=False)
                moves.append((f"posts request {g.posted}", g2, "run"))
            consumed = g.completed
            if consumed == requests:
                moves.append(("reads the last completions: done", _set(g, consumed=consumed), None))
            else:
                g2 = _set(g, consumed=consumed)
                if relaunch_on_poll and not g.running and g.posted > consumed:
                    moves.append(("poll: loop ended with work left, launches it",
                                  _set(g2, running=True, armed=False), "run"))
                elif g2 != g:
                    moves.append(("poll: reads completions", g2, "run"))
        return moves

    def device(g, pc, trace):
        if pc == "leaving":
            return [("leaves", _set(g, running=False, armed=False), "loop")]
        if not g.running:
            return [("done", g, None)] if g.completed == requests else []
        moves = []
        if g.posted > g.taken:
            moves.append(("takes a request", _set(g, taken=g.taken + 1, active=g.active + 1, armed=False), "loop"))
        if g.active > 0:
            moves.append(("completes a request", _set(g, active=g.active - 1, completed=g.completed + 1,
                                                      armed=False), "loop"))
        if g.active == 0 and g.posted == g.taken:
            if not g.armed:
                moves.append(("nothing to do: arms the idle limit", _set(g, armed=True), "loop"))
            else:
                moves.append(("idle limit passed, ring empty: decides to leave", g, "leaving"))
        return moves

    def final(g, trace):
        if g.completed != requests or g.consumed != requests:
            raise Violation(f"{g.completed} of {requests} requests completed, {g.consumed} read", trace)

    g0 = LoopState(posted=0, taken=0, active=0, completed=0, consumed=0, running=True, armed=False)
    return (g0, ("run", "loop")), [host, device], final


# --------------------------------------------------------------------------
# the bulk delete's ticketed turn at node 0

TurnState = namedtuple("TurnState", "ticket serving holder order")


def delete_turn_model(blocks=3, rounds=2, pass_after_lock=True, take_ticket=True):
    """The ticketed turn of a bulk delete's blocks at node 0
    (include/gpuheap_device.cuh `takeTurn`, `deleteRootImpl` with fair):
    thread 0 draws t = atomicAdd(delTicket), waits until delServing == t,
    locks node 0 (a CAS on its lock word, retried while it is held), then
    passes the turn (delServing = t + 1) and, after its root step, unlocks
    node 0.  Each block deletes `rounds` times.

    Invariants: node 0 is held by one block at a time, and blocks take it in
    ticket order -- the fairness the ticket is for (racing on the lock word
    let one block lose for a whole delete phase).  Planted mistakes: passing
    the turn before the lock is held (the next ticket then races the lock),
    and no tickets at all (every block races on the lock word)."""

    def block(i):
        def act(g, pc, trace):
            step = pc[0]
            r = pc[1]
            nxt_round = ("draw", r + 1) if r + 1 < rounds else None
            if step == "draw":
                if not take_ticket:
                    return [("races for node 0", g, ("lock", r, None))]
                return [(f"draws ticket {g.ticket}", _set(g, ticket=g.ticket + 1), ("wait", r, g.ticket))]
            t = pc[2]
            if step == "wait":
                if g.serving != t:
                    return []
                if pass_after_lock:
                    return [(f"ticket {t} served", g, ("lock", r, t))]
                return [(f"ticket {t} served, passes the turn at once", _set(g, serving=t + 1), ("lock_only", r, t))]
            if step in ("lock", "lock_only"):
                if g.holder != -1:
                    return []  # the CAS fails: retry
                g2 = _set(g, holder=i, order=g.order + ((t if t is not None else i),))
                if step == "lock" and t is not None:
                    return [("locks node 0", g2, ("pass", r, t))]
                return [("locks node 0", g2, ("unlock", r, t))]
            if step == "pass":
                return [(f"passes the turn to {t + 1}", _set(g, serving=t + 1), ("unlock", r, t))]
            if step == "unlock":
                return [("root step done, unlocks node 0", _set(g, holder=-1), nxt_round)]
            return []
        act.__name__ = f"b{i}"
        return act

    def final(g, trace):
        if take_ticket and list(g.order) != sorted(g.order):
            raise Violation(f"node 0 taken in ticket order {list(g.order)}", trace)
        if len(g.order) != blocks * rounds:
            raise Violation(f"{len(g.order)} root steps of {blocks * rounds}", trace)

    g0 = TurnState(ticket=0, serving=0, holder=-1, order=())
    return (g0, tuple(("draw", 0) for _ in range(blocks))), [block(i) for i in range(blocks)], final


# --------------------------------------------------------------------------
# top-down reserved bulk inserts: the root in target order

ResvState = namedtuple("ResvState", "status turn written")


def reserved_insert_model(targets=5, use_turn=True, pass_after_root=True):
    """Top-down bulk inserts into reserved targets (include/gpuheap_device.cuh
    `insertionReserved`, `insert_topdown` with reserved, `waitTurn`;
    gpuheap_gb300/csrc/heap_kernels.cuh `k_reserve`, `k_mark_reserved`):
    targets 1..`targets` are drawn at once and their lock words set to
    TARGET; insert t waits until resvTurn == t, locks the root (node 1;
    insert 1's target is the root itself), passes the turn (resvTurn = t +
    1), then walks its path hand over hand -- it locks the next node
    (waiting while it is INUSE or still an earlier insert's TARGET) before
    it frees the current one -- and at its target swaps TARGET for INUSE,
    writes it and frees it.

    Invariants: every target is written once, by its insert, and nobody
    waits forever.  A walk that meets an earlier insert's unwritten target
    waits there while holding an ancestor; the earlier insert needs that
    ancestor too, so the root must be taken in target order.  Planted
    mistakes: no turn (inserts race for the root), and the turn passed
    before the root is held."""

    def path(t):
        p = []
        x = t
        while x >= 1:
            p.append(x)
            x >>= 1
        return list(reversed(p))  # 1 .. t

    def ins(t):
        P = path(t)

        def act(g, pc, trace):
            step = pc[0]
            if step == "turn":
                if use_turn and g.turn != t:
                    return []
                if t == 1 or not pass_after_root:
                    g2 = _set(g, turn=t + 1) if use_turn else g
                    return [("turn: passes it on" if use_turn else "no turn", g2,
                             ("at", 0) if t == 1 else ("root", 0))]
                return [("turn", g, ("root", 0))]
            if step == "root":
                if g.status[1] != TD_AVAIL:
                    return []
                g2 = _set(g, status=_put(g.status, 1, TD_INUSE))
                if use_turn and pass_after_root:
                    g2 = _set(g2, turn=t + 1)
                return [("locks the root" + (", passes the turn" if use_turn and pass_after_root else ""), g2,
                         ("at", 0))]
            if step == "at":
                k = pc[1]
                cur = P[k]
                if cur == t:
                    if g.status[t] != TD_TARGET:
                        raise Violation(f"insert {t} found its target in state {g.status[t]}",
                                        list(trace) + [f"i{t}:at target"])
                    return [("writes its target", _set(g, status=_put(g.status, t, TD_AVAIL),
                                                      written=g.written + (t,)), None)]
                nxt = P[k + 1]
                if nxt != t:
                    if g.status[nxt] != TD_AVAIL:
                        return []
                    st = _put(_put(g.status, nxt, TD_INUSE), cur, TD_AVAIL)
                    return [(f"locks {nxt}, frees {cur}", _set(g, status=st), ("at", k + 1))]
                return [(f"frees {cur}, on to its target", _set(g, status=_put(g.status, cur, TD_AVAIL)),
                         ("at", k + 1))]
            return []
        act.__name__ = f"i{t}"
        return act

    def final(g, trace):
        if sorted(g.written) != list(range(1, targets + 1)):
            raise Violation(f"targets written {g.written}", trace)
        if any(s != TD_AVAIL for s in g.status[1:]):
            raise Violation(f"lock words left {g.status[1:]}", trace)

    g0 = ResvState(status=(TD_AVAIL,) + (TD_TARGET,) * targets, turn=1, written=())
    return (g0, tuple(("turn",) for _ in range(targets))), [ins(t) for t in range(1, targets + 1)], final


# --------------------------------------------------------------------------
# the retrieving heap's auxiliary buffer

AuxState = namedtuple("AuxState", "buf lock heap done")


def aux_buffer_model(blocks=2, count=2, buffered=(3,), heap_keys=(10, 11, 12, 14), reread_after_relock=True):
    """gh::RetHeapAux::retrieve (include/gpuheap_retrieve.cuh; reference
    applications/sssp_longfei_new/heap_with_aux.cuh:48-119): under the
    buffer's lock a block takes the newest `count` buffered entries, or all
    of them and then -- with the lock released -- the rest from the heap;
    it locks again, hands every entry to the check, and appends the ones
    with work left (here: the even ones) after the buffer's current end.

    Every entry must end in exactly one place: the buffer, the heap, or
    handed out for good.  Planted mistake: appending after the end the
    block saw before it released the lock, instead of reading it again
    (another block's entries appended in between are overwritten)."""
    work_left = lambda e: e % 2 == 0

    def block(i):
        def act(g, pc, trace):
            step = pc[0]
            if step == "lock":
                if g.lock != -1:
                    return []
                return [("locks the buffer", _set(g, lock=i), ("take",))]
            if step == "take":
                have = len(g.buf)
                if have > count:
                    got = g.buf[have - count:]
                    return [(f"takes the newest {got}", _set(g, buf=g.buf[:have - count]), ("check", got, have - count))]
                got = g.buf
                if count - have > 0:
                    return [(f"takes all {got}, unlocks for the heap", _set(g, buf=(), lock=-1), ("heap", got))]
                return [(f"takes all {got}", _set(g, buf=()), ("check", got, 0))]
            if step == "heap":
                got = pc[1]
                want = count - len(got)
                more = g.heap[:want]
                return [(f"retrieves {more} from the heap", _set(g, heap=g.heap[want:]), ("relock", got + more, len(g.buf)))]
            if step == "relock":
                if g.lock != -1:
                    return []
                end = len(g.buf) if reread_after_relock else 0
                return [("locks the buffer again", _set(g, lock=i), ("check", pc[1], end))]
            if step == "check":
                got, end = pc[1], pc[2]
                back = tuple(e for e in got if work_left(e))
                buf = g.buf[:end] + back  # appended after `end`, overwriting what lies there
                lost = set(g.buf[end:]) - set(back)
                if lost:
                    # entries of another block are overwritten
                    raise Violation(f"block {i} appended at {end} over entries {sorted(lost)}",
                                    list(trace) + [f"b{i}:append"])
                done = g.done + tuple(e for e in got if not work_left(e))
                return [(f"hands out {got}, buffers {back} again", _set(g, buf=buf, done=done, lock=-1), None)]
            return []
        act.__name__ = f"b{i}"
        return act

    def final(g, trace):
        places = list(g.buf) + list(g.heap) + list(g.done)
        if sorted(places) != sorted(buffered + heap_keys):
            raise Violation(f"entries end as buffer {g.buf}, heap {g.heap}, out {g.done}", trace)

    g0 = AuxState(buf=tuple(buffered), lock=-1, heap=tuple(heap_keys), done=())
    return (g0, tuple(("lock",) for _ in range(blocks))), [block(i) for i in range(blocks)], final


# --------------------------------------------------------------------------
# the FIFO's whole-call push: the grid copies, the last block publishes

BulkState = namedtuple("BulkState", "slots arrived write got")


def fifo_bulk_model(blocks=3, last_commits=True, arrive_after_copy=True):
    """k_fifo_bulk_push (gpuheap_gb300/csrc/fifo.cu): one thread reserved
    positions [0, blocks); block b copies position b, then thread 0 fences
    and counts itself in (atomicAdd on bulkDone); the block that counts
    last publishes write = blocks.  A popper reads every position below
    `write` as soon as it sees it.

    Invariant: a position the popper reads is written.  Planted mistakes:
    the first block to count in publishes, and a block that counts in
    before its copy."""

    def block(b):
        def act(g, pc, trace):
            if pc == "copy":
                slots = _put(g.slots, b, True)
                return [(f"copies position {b}", _set(g, slots=slots), "arrive" if arrive_after_copy else None)]
            if pc == "arrive":
                n = g.arrived + 1
                last = n == blocks if last_commits else n == 1
                return [(f"counts in ({n})", _set(g, arrived=n), "commit" if last else None)]
            if pc == "commit":
                return [("publishes write", _set(g, write=blocks), None)]
            if pc == "arrive_first":
                n = g.arrived + 1
                last = n == blocks
                return [(f"counts in ({n}) before its copy", _set(g, arrived=n), ("copy_then", last))]
            if isinstance(pc, tuple) and pc[0] == "copy_then":
                slots = _put(g.slots, b, True)
                if pc[1]:
                    return [(f"copies position {b}", _set(g, slots=slots), "commit")]
                return [(f"copies position {b}", _set(g, slots=slots), None)]
            return []
        act.__name__ = f"b{b}"
        return act

    def popper(g, pc, trace):
        k = pc
        if k >= g.write:
            return [] if g.write < blocks else [("done", g, None)]
        if not g.slots[k]:
            raise Violation(f"popper read position {k} before its block copied it", list(trace) + [f"pop:read {k}"])
        return [(f"reads position {k}", _set(g, got=g.got + 1), k + 1 if k + 1 < blocks else None)]

    def final(g, trace):
        if g.got != blocks or g.write != blocks:
            raise Violation(f"popper read {g.got} of {blocks} (write {g.write})", trace)

    g0 = BulkState(slots=(False,) * blocks, arrived=0, write=0, got=0)
    start = "copy" if arrive_after_copy else "arrive_first"
    return (g0, tuple(start for _ in range(blocks)) + (0,)), [block(b) for b in range(blocks)] + [popper], final
