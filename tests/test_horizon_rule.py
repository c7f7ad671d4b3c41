"""The closed form the warp and large-polytope EPA tiers use for the horizon, against the
reference's sequential PushEdge (code/nans.cpp:232-266): a pushed edge cancels the FIRST stored
edge that is its reverse (vertex equality compares positions; a NaN position equals nothing),
else it is appended. The closed form decides each push from its group (the unordered pair of
canonical vertex ids) alone: the survivors of a group are the last (#majority - #minority)
pushes of the majority orientation; in a self-loop group (both ends equal) the last push
survives iff the group has an odd number of pushes; a push with a NaN end always survives.
Survivors keep push order. Pure CPU."""
import random

NAN = -1  # canonical id of a vertex with a NaN coordinate


def sequential(pushes):
    stored = []
    for k, (u, v) in enumerate(pushes):
        hit = -1
        if u != NAN and v != NAN:
            for e, (x, y, _) in enumerate(stored):
                if x == v and y == u:
                    hit = e
                    break
        if hit >= 0:
            stored.pop(hit)
        else:
            stored.append((u, v, k))
    return [k for _, _, k in stored]


def closed_form(pushes):
    out = []
    for k, (u, v) in enumerate(pushes):
        if u == NAN or v == NAN:
            out.append(k)
            continue
        key, d = (min(u, v), max(u, v)), u > v
        same = opp = after = 0
        for j, (a, b) in enumerate(pushes):
            if a == NAN or b == NAN or (min(a, b), max(a, b)) != key:
                continue
            if (a > b) == d:
                same += 1
                after += j > k
            else:
                opp += 1
        if u == v:
            alive = after == 0 and same % 2 == 1
        else:
            alive = same > opp and after < same - opp
        if alive:
            out.append(k)
    return out


def test_closed_form_equals_sequential_push_edge():
    rng = random.Random(7)
    for _ in range(20000):
        ids = rng.randint(1, 4)
        pushes = []
        for _ in range(rng.randint(1, 12)):
            u = NAN if rng.random() < 0.05 else rng.randrange(ids)
            v = NAN if rng.random() < 0.05 else rng.randrange(ids)
            pushes.append((u, v))
        assert closed_form(pushes) == sequential(pushes), pushes


def test_closed_form_on_a_polytope_horizon():
    # two visible triangles sharing the edge (1, 2): the shared edge cancels, the other four
    # edges form the horizon in push order
    pushes = [(0, 1), (1, 2), (2, 0), (2, 1), (1, 3), (3, 2)]
    assert sequential(pushes) == closed_form(pushes) == [0, 2, 4, 5]
