"""Test helper: the oracle's paint record for a product paint object."""
from oracle import oracle as O
from rasterize_gb300.paint import GradLinear, GradRadial, LinColor


def oracle_paint(p):
    if isinstance(p, LinColor):
        return O.make_paint(kind=0, solid=p.rgba())
    stops = [(s.position, s.color.rgba()) for s in p.stops]
    if isinstance(p, GradLinear):
        return O.make_paint(kind=1, units=int(p.units), spread=int(p.spread), linear_colors=p.linear_colors,
                            tr=p.tr, p0=p.start, p1=p.end, stops=stops)
    if isinstance(p, GradRadial):
        return O.make_paint(kind=2, units=int(p.units), spread=int(p.spread), linear_colors=p.linear_colors,
                            tr=p.tr, p0=p.center, p1=p.fcenter, r0=p.radius, r1=p.fradius, stops=stops)
    raise TypeError(p)


def oracle_scene(sc, width, height, bg=(0, 0, 0, 0)):
    paths = [f[0] for f in sc.fills]
    trs = [f[1] for f in sc.fills]
    rules = [f[2] for f in sc.fills]
    paints = [oracle_paint(f[3]) for f in sc.fills]
    return O.scene_render(paths, trs, rules, paints, width, height, bg=bg)


def oracle_tree(sc):
    """The oracle's nested-tuple form of a product Scene tree."""
    if isinstance(sc, tuple):
        path, tr, rule, paint = sc
        return ("fill", path, tr, int(rule), oracle_paint(paint))
    if sc.kind == "group":
        return ("group", [oracle_tree(c) for c in sc.children])
    if sc.kind == "opacity":
        return ("opacity", oracle_tree(sc.children[0]), sc.params["opacity"])
    if sc.kind == "transform":
        return ("transform", oracle_tree(sc.children[0]), sc.params["tr"])
    if sc.kind == "stroke":
        st = sc.params["style"]
        return ("stroke", sc.params["path"], sc.params["tr"],
                (st.width, int(st.line_join), st.miter_limit, int(st.line_cap)), oracle_paint(sc.params["paint"]))
    return ("clip", oracle_tree(sc.children[0]), sc.params["path"], int(sc.params["units"]), int(sc.params["rule"]))


def oracle_scene_tree(sc, width, height, bg=(0, 0, 0, 0)):
    return O.scene_tree_render(oracle_tree(sc), width, height, bg=bg)
