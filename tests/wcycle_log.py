"""The reference's cycle tables of stdout0.out (elliptic::Print_Pre_Cycle /
Print_Post_Cycle, src/output.cc:1355-1605) rendered from a list of
(level, post, cycle, norm) calls: a header and a rule before the top level's
pre-smoothing line, a rule and `norm  -->  eps` after its post-smoothing
line, one indented `|Loo[k] : norm` line per call."""


def render_cycle_tables(events, nlevels, eps):
    top = nlevels - 1
    rule = "=" * 24 * (top + 1) + "\n"
    out = []
    for k, post, cycle, norm in events:
        if not post and k == top:
            out.append("\n\nCycle: %d\n" % cycle + rule)
        out.append("|\t\t\t" * k + "|Loo[%d] : %.8e" % (k, norm) + "|\t\t\t" * (top + 1 - k) + "\n")
        if post and k == top:
            out.append(rule + "%.8e  -->  %.8e\n" % (norm, eps))
    return "".join(out)


def check_wcycle_calls(events, nlevels, tol):
    """Asserts that (level, post, cycle, norm) calls are those of one
    elliptic::Wcycle top-level call (src/elliptic.cc:1468-1968): level k
    repeats [pre k, (the coarsest solve | level k-1's own loop), post k] from
    the caller's cycle number, one more each time, until its post norm is
    <= tol; every call of one iteration prints the iteration's number.
    Returns the number of iterations of each level."""
    pos = 0
    iters = [0] * nlevels

    def take(level, post, cycle):
        nonlocal pos
        assert pos < len(events), ("missing call", level, post, cycle)
        e = events[pos]
        assert (e[0], e[1], e[2]) == (level, post, cycle), (pos, e, (level, post, cycle))
        pos += 1
        return e[3]

    def level_loop(k, icycle):
        c = icycle
        while True:
            take(k, 0, c)
            if k == 1:
                take(0, 0, c)
            else:
                level_loop(k - 1, c)
            norm = take(k, 1, c)
            iters[k] += 1
            c += 1
            if not norm > tol:
                return

    level_loop(nlevels - 1, 0)
    assert pos == len(events), ("extra calls", events[pos:pos + 3])
    return iters
