"""Race detection for the path's lock-free protocols, on CPU: every
interleaving of the atomic steps of the bottom-up park protocol, the
top-down target hand-off, the FIFO ring, the searches' termination
protocol, the retrieving heap's steal and the owner-mode delete's lends
(oracle/lock_model.py) keeps its invariants and never deadlocks,
and the explorer finds each planted mistake -- the ones these protocols
exist to prevent -- with the interleaving that exposes it."""
import pytest

from oracle import lock_model as lm


def _run(model):
    init, actors, final = model
    return lm.explore(init, actors, final)


@pytest.mark.parametrize("with_taker", [True, False])
@pytest.mark.parametrize("with_passer", [True, False])
def test_ticketed_parks_are_safe(with_taker, with_passer):
    """The device protocol: tickets unique per insert, trust on finding
    one's own ticket, DELMOD after a pass-through."""
    r = _run(lm.bottomup_park_model(with_taker=with_taker, with_passer=with_passer))
    assert r.finals >= 1 and not r.deadlocks


def test_reference_parks_are_safe_without_trust():
    """The reference's protocol: one INSHOLD value, and the node is always
    read back from memory (heap/buitdd/heap.cuh:643-673)."""
    r = _run(lm.bottomup_park_model(tagged=False, trust_own_park=False))
    assert r.finals >= 1 and not r.deadlocks


def test_untagged_parks_with_trust_are_caught():
    """Trusting INSHOLD without tickets loses a batch: a deleter takes the
    parked node as its last node, a new insert claims it and parks there
    too, and the first insert finds 'its' park value again."""
    with pytest.raises(lm.Violation) as e:
        _run(lm.bottomup_park_model(tagged=False, with_passer=False))
    trace = e.value.trace
    assert any(t.startswith("taker:take last x") for t in trace)
    assert any(t.startswith("ins2:cas p fail; park x") for t in trace)
    assert trace[-1].endswith("retake")


def test_restoring_the_ticket_after_a_pass_through_is_caught():
    """A deleter that passed through a parked node must leave DELMOD, not
    the ticket it found (gpuheap_device.cuh tryChild)."""
    with pytest.raises(lm.Violation) as e:
        _run(lm.bottomup_park_model(delmod_on_release=False))
    assert any("release x as" in t and "as 2" not in t for t in e.value.trace)


@pytest.mark.parametrize("steps", [0, 1, 2, 4])
@pytest.mark.parametrize("check_on_path", [True, False])
def test_topdown_handoff_is_safe(steps, check_on_path):
    """The batch reaches the deleter exactly once and t ends AVAIL, whether
    the insert sees the mark on its path or at its final CAS -- the path
    check only shortens the deleter's wait."""
    r = _run(lm.topdown_handoff_model(path_steps=steps, check_marked_on_path=check_on_path))
    assert r.finals == 1 and not r.deadlocks


def test_topdown_plain_store_at_the_target_deadlocks():
    """Writing t with a plain store ignores a mark set after the last path
    check: the deleter then waits forever for the hand-over."""
    r = _run(lm.topdown_handoff_model(cas_at_target=False))
    assert r.deadlocks
    dl = r.deadlocks[0]
    assert "dele:cas t TARGET->MARKED" in dl and "ins:store t INUSE (no cas)" in dl


def test_topdown_reading_the_root_before_the_handoff_is_caught():
    with pytest.raises(lm.Violation, match="before the hand-over"):
        _run(lm.topdown_handoff_model(wait_for_handoff=False))


def test_explorer_reports_deadlock_and_final_states():
    """The explorer itself: two actors that each wait for the other's flag
    deadlock; one that sets a flag first lets the other finish."""
    from collections import namedtuple
    S = namedtuple("S", "a b")

    def first(g, pc, trace):
        if pc == 0:
            return [("wait b", g, 1)] if g.b else []
        return [("set a", S(True, g.b), None)] if pc == 1 else []

    def second(g, pc, trace):
        if pc == 0:
            return [("wait a", g, 1)] if g.a else []
        return [("set b", S(g.a, True), None)] if pc == 1 else []

    r = lm.explore((S(False, False), (0, 0)), [first, second])
    assert r.deadlocks == [[]] and r.finals == 0
    r = lm.explore((S(False, True), (0, 0)), [first, second])
    assert not r.deadlocks and r.finals == 1


@pytest.mark.parametrize("blocks,depth", [(2, 2), (3, 2), (2, 3)])
def test_termination_protocol_ends_exactly_when_work_is_done(blocks, depth):
    """worklist.cuh: in every interleaving each block leaves, and only once
    every unit of the work tree was taken, the heap is empty and busy is 0."""
    r = _run(lm.termination_model(blocks=blocks, depth=depth))
    assert r.finals == 1 and not r.deadlocks


def test_waiting_blocks_counted_busy_never_end():
    """Planted: a waiting block that counts itself busy keeps the others
    waiting forever once the work runs out."""
    r = _run(lm.termination_model(count_while_waiting=True))
    assert r.deadlocks and r.finals == 0
    assert all("count self while waiting" in t for t in r.deadlocks[0][-2:])


@pytest.mark.parametrize("pushes,pops,capacity", [((1, 1, 1), (1, 1, 1), 2), ((2, 1), (1, 2), 2),
                                                   ((1, 1, 1), (2, 1), 1), ((2, 2), (3, 1), 2)])
def test_fifo_protocol_is_safe(pushes, pops, capacity):
    """gpuheap_fifo.cuh on a ring that wraps (down to one slot): no slot is
    read before its push wrote it or after a later push overwrote it, every
    key comes out once, and no interleaving leaves a block waiting."""
    r = _run(lm.fifo_model(pushes=pushes, pops=pops, capacity=capacity))
    assert r.finals >= 1 and not r.deadlocks


@pytest.mark.parametrize("mistake,found", [("wait_room", "found (2, 2)"), ("publish_in_order", "found (-1, -1)"),
                                           ("claim_by_cas", "found"), ("free_in_order", "found")])
def test_fifo_planted_mistakes_are_caught(mistake, found):
    """Each of the four waits and checks is needed: without the room wait a
    push overwrites an unread slot, publishing out of order exposes an
    unwritten one, a plain-store claim hands a position to two pops, and
    freeing out of order lets a push overwrite a slot still being copied."""
    with pytest.raises(lm.Violation, match="popper read slot") as e:
        _run(lm.fifo_model(**{mistake: False}))
    assert found in str(e.value)


def test_waiting_for_the_parent_without_parking_deadlocks():
    """Inserts lock child then parent, sifting deleters parent then child:
    an insert that waits for its parent while still holding its node
    deadlocks against a deleter passing through (the park breaks the cycle);
    with no deleter passing, the same insert finishes."""
    r = _run(lm.bottomup_park_model(park_before_wait=False, with_taker=False))
    assert r.deadlocks and r.deadlocks[0] == ["holder:sift toward x", "ins:cas p fail; wait holding x"]
    r = _run(lm.bottomup_park_model(park_before_wait=False, with_taker=False, with_passer=False))
    assert not r.deadlocks and r.finals == 1


# ------------------------------------------------------ retrieving heap steal
@pytest.mark.parametrize("steps", [1, 2, 3])
def test_retrieve_steal_is_safe(steps):
    res = _run(lm.retrieve_steal_model(path_steps=steps))
    assert res.deadlocks == [] and res.finals > 0


@pytest.mark.parametrize("mistake", ["lock_before_check", "retrieve_locks_target", "root_before_signal"])
def test_retrieve_steal_planted_mistakes_are_caught(mistake):
    try:
        res = _run(lm.retrieve_steal_model(path_steps=2, **{mistake: False}))
    except lm.Violation:
        return
    assert res.deadlocks, f"{mistake}: no violation and no deadlock found"


# ------------------------------------------------ owner-mode lend and return
@pytest.mark.parametrize("deletes,nodes", [(2, 1), (3, 1), (3, 2), (4, 2), (5, 3)])
def test_owner_lend_round_trip_is_safe(deletes, nodes):
    """The owner lends a level-R node with the carried batch, the worker's
    first level rewrites it and leaves kLentBack, the returner reloads it:
    every plan reads the node's current version, no reload lands during a
    pass, every carried batch reaches its own lend."""
    res = _run(lm.owner_lend_model(deletes=deletes, nodes=nodes))
    assert res.deadlocks == [] and res.finals == 1


@pytest.mark.parametrize("mistake,found", [
    ("mark_after_pass", "lands while the pass reads"),
    ("back_after_write", "slots at"),
    ("returner_checks_status", "lock words"),
    ("cons_after_load", "carried batch for lend"),
    ("lender_waits_cons", "carried batch for lend"),
])
def test_owner_lend_planted_mistakes_are_caught(mistake, found):
    with pytest.raises(lm.Violation) as e:
        _run(lm.owner_lend_model(deletes=4, nodes=2, **{mistake: False}))
    assert found in str(e.value)


@pytest.mark.parametrize("lends", [(True, False, True, True), (True,) * 5, (False,) * 4, (False, True, True, False, True)])
def test_owner_carried_buffers_are_safe(lends):
    """The taker loads the next delete's last node into the other buffer;
    a buffer is loaded again only after its delete and, when it lent, the
    lender's copy are done."""
    res = _run(lm.owner_taker_model(deletes=len(lends), lends=lends))
    assert res.deadlocks == [] and res.finals == 1


@pytest.mark.parametrize("mistake,found", [
    ("taker_waits_free", "while it is read"),
    ("free_after_copy", "while it is read"),
    ("compute_waits_ready", "holding delete"),
])
def test_owner_carried_buffer_mistakes_are_caught(mistake, found):
    with pytest.raises(lm.Violation) as e:
        _run(lm.owner_taker_model(**{mistake: False}))
    assert found in str(e.value)


# ------------------------------------------------ served loop's token queue
@pytest.mark.parametrize("blocks,query_blocks,cells,stints", [(2, 2, 2, 3), (3, 2, 2, 2), (2, 3, 3, 2)])
def test_serve_token_queue_is_safe(blocks, query_blocks, cells, stints):
    """Every pop reads its own position's token, the query completes once
    after all its tokens retired, the ring ends empty, nobody waits forever."""
    res = _run(lm.serve_token_model(blocks=blocks, query_blocks=query_blocks, cells=cells, max_stints=stints))
    assert res.deadlocks == [] and res.finals >= 1


@pytest.mark.parametrize("mistake,found", [
    ("pop_by_cas", "tokens out"),
    ("push_waits_cell", "read position"),
    ("release_after_read", "read position"),
])
def test_serve_token_queue_mistakes_are_caught(mistake, found):
    with pytest.raises(lm.Violation) as e:
        _run(lm.serve_token_model(**{mistake: False}))
    assert found in str(e.value)


def test_serve_retire_by_load_and_store_loses_the_completion():
    """Two blocks retire the last two tokens by load and store: both write
    1, nobody completes the query and every block waits on an empty ring."""
    res = _run(lm.serve_token_model(retire_atomic=False))
    assert res.deadlocks
    assert any(t.startswith("b0:reads tokens 2") or t.startswith("b1:reads tokens 2") for t in res.deadlocks[0])


# ------------------------------------------------ served loop's host rings
@pytest.mark.parametrize("queries,cap,completers", [(4, 2, 2), (5, 2, 2), (4, 3, 3)])
def test_serve_rings_are_safe(queries, cap, completers):
    """Requests out through pinned memory, completions back in any order of
    ending: every record is read as written, none is overwritten unread."""
    res = _run(lm.serve_rings_model(queries=queries, cap=cap, completers=completers))
    assert res.deadlocks == [] and res.finals >= 1


@pytest.mark.parametrize("mistake,found", [
    ("guard_by_completions", "before the host read it"),
    ("seq_after_fields", "host read completion"),
])
def test_serve_rings_mistakes_are_caught(mistake, found):
    with pytest.raises(lm.Violation) as e:
        _run(lm.serve_rings_model(**{mistake: False}))
    assert found in str(e.value)


def test_serve_rings_taken_is_advisory():
    """The host reuses a request record only after its completion, so the
    device may publish `taken` before its copy without harm."""
    res = _run(lm.serve_rings_model(take_after_copy=False))
    assert res.deadlocks == [] and res.finals >= 1


# ------------------------------------------------ progress (livelock) check
@pytest.mark.parametrize("name", ["bottomup", "topdown", "termination", "retrieve", "fifo", "lend", "taker",
                                  "tokens", "tokens_spin", "rings"])
def test_every_state_can_finish(name):
    """Beyond deadlocks: from every reachable state of each protocol some
    interleaving still finishes, so no cycle of moves can run forever."""
    model = {
        "bottomup": lambda: lm.bottomup_park_model(),
        "topdown": lambda: lm.topdown_handoff_model(),
        "termination": lambda: lm.termination_model(),
        "retrieve": lambda: lm.retrieve_steal_model(),
        "fifo": lambda: lm.fifo_model(),
        "lend": lambda: lm.owner_lend_model(deletes=4, nodes=2),
        "taker": lambda: lm.owner_taker_model(),
        "tokens": lambda: lm.serve_token_model(),
        "tokens_spin": lambda: lm.serve_token_model(poll_is_wait=False),
        "rings": lambda: lm.serve_rings_model(),
    }[name]()
    init, actors, final = model
    res = lm.explore(init, actors, final, progress=True)
    assert res.finals >= 1 and not res.deadlocks and not res.stuck, res.stuck[:1]


def test_spinning_retire_by_load_and_store_is_a_livelock():
    """With the device's spinning poll, the lost completion is no deadlock:
    the blocks keep polling an empty ring.  Only the progress check sees
    that no state after the lost write can finish."""
    init, actors, final = lm.serve_token_model(retire_atomic=False, poll_is_wait=False)
    res = lm.explore(init, actors, final, progress=True)
    assert not res.deadlocks and res.stuck
    assert any("reads tokens 2" in t for t in res.stuck[0])


@pytest.mark.parametrize("requests", [1, 2, 3])
def test_serve_loop_relaunch_never_strands_a_request(requests):
    """The loop may leave on its idle limit at any time the ring looked
    empty; the host's poll launches it again while requests are
    outstanding, so every request completes from every state."""
    init, actors, final = lm.serve_loop_model(requests=requests)
    res = lm.explore(init, actors, final, progress=True)
    assert res.finals >= 1 and not res.deadlocks and not res.stuck


def test_serve_loop_relaunch_only_on_post_strands_a_request():
    init, actors, final = lm.serve_loop_model(relaunch_on_poll=False)
    res = lm.explore(init, actors, final, progress=True)
    assert res.stuck and res.deadlocks
    t = res.deadlocks[0]
    assert "device:idle limit passed, ring empty: decides to leave" in t and t[-1] == "device:leaves"


# ------------------------------------------------ bulk delete's ticketed turn
@pytest.mark.parametrize("blocks,rounds", [(2, 2), (3, 2), (4, 2)])
def test_delete_turn_is_fifo(blocks, rounds):
    """Blocks take node 0 in ticket order, one at a time, and never wait forever."""
    init, actors, final = lm.delete_turn_model(blocks=blocks, rounds=rounds)
    res = lm.explore(init, actors, final, progress=True)
    assert res.finals == 1 and not res.deadlocks and not res.stuck


def test_delete_turn_passed_before_the_lock_breaks_the_order():
    with pytest.raises(lm.Violation, match="ticket order"):
        _run(lm.delete_turn_model(pass_after_lock=False))


def test_delete_without_tickets_lets_a_block_lose_every_race():
    """Racing on the lock word alone: there are runs in which block 0 takes
    node 0 only after every other block has finished all its rounds."""
    orders = []
    init, actors, _ = lm.delete_turn_model(take_ticket=False)
    lm.explore(init, actors, lambda g, trace: orders.append(g.order))
    assert any(o[-2:] == (0, 0) and 0 not in o[:-2] for o in orders)


# ------------------------------------------------ top-down reserved inserts
@pytest.mark.parametrize("targets", [3, 5, 7])
def test_reserved_topdown_inserts_finish(targets):
    """Reserved targets entered in target order: every target is written
    once, from every state the inserts can finish."""
    init, actors, final = lm.reserved_insert_model(targets=targets)
    res = lm.explore(init, actors, final, progress=True)
    assert res.finals >= 1 and not res.deadlocks and not res.stuck


@pytest.mark.parametrize("mistake", [dict(use_turn=False), dict(pass_after_root=False)])
def test_reserved_topdown_inserts_out_of_order_deadlock(mistake):
    """A later target's walk holds an ancestor while it waits at an earlier
    insert's unwritten target, which needs that ancestor: the root must be
    entered in target order, and the turn passed only once it is held."""
    init, actors, final = lm.reserved_insert_model(**mistake)
    res = lm.explore(init, actors, final, progress=True)
    assert res.deadlocks and res.stuck


# ------------------------------------------------ retrieving heap's aux buffer
@pytest.mark.parametrize("blocks,buffered,heap_keys", [(2, (3,), (10, 11, 12, 14)), (3, (3, 4), (10, 11, 12, 13, 14, 16)),
                                                       (2, (2, 3), (10, 11, 12))])
def test_aux_buffer_keeps_every_entry(blocks, buffered, heap_keys):
    """Entries taken, handed to the check and buffered again under the
    lock (released while the heap is read): each ends in one place."""
    init, actors, final = lm.aux_buffer_model(blocks=blocks, buffered=buffered, heap_keys=heap_keys)
    res = lm.explore(init, actors, final, progress=True)
    assert res.finals >= 1 and not res.deadlocks and not res.stuck


def test_aux_buffer_stale_end_overwrites_entries():
    """Appending at the end seen before the heap read loses the entries
    another block appended meanwhile."""
    with pytest.raises(lm.Violation, match="appended at 0 over entries"):
        _run(lm.aux_buffer_model(reread_after_relock=False))


# ------------------------------------------------ FIFO whole-call publish
@pytest.mark.parametrize("blocks", [2, 3, 4])
def test_fifo_bulk_publish_after_every_copy(blocks):
    init, actors, final = lm.fifo_bulk_model(blocks=blocks)
    res = lm.explore(init, actors, final, progress=True)
    assert res.finals == 1 and not res.deadlocks and not res.stuck


@pytest.mark.parametrize("mistake", [dict(last_commits=False), dict(arrive_after_copy=False)])
def test_fifo_bulk_early_publish_is_caught(mistake):
    with pytest.raises(lm.Violation, match="before its block copied it"):
        _run(lm.fifo_bulk_model(**mistake))
