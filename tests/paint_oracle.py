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
