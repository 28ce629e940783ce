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
