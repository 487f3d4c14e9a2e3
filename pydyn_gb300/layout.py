"""The declared bounds of every state array of a region, as TM5 declares them and pydyn's
ZoomState holds them (pydyn zoom/state.py:13-50, layout.py:26-36):

    m (-1:im+2, -1:jm+2, 1:lm)        rm rxm rym rzm (-1:im+2, -1:jm+2, 1:lm, 1:nt)
    am bm cm (0:im+1, 0:jm+1, 0:lm+1) pu (0:im, 1:jm, 1:lm)   pv (1:im, 1:jm+1, 1:lm)
    sp (-1:im+2, -1:jm+2, 1:1)        phlb (-1:im+2, -1:jm+2, 1:lm+1)   dxyp (1:jm)

Pure host description (the input generator and the device state both read it)."""

FIELDS = ("m", "rm", "rxm", "rym", "rzm", "am", "bm", "cm", "pu", "pv", "sp", "phlb", "dxyp")
TRACERS = ("rm", "rxm", "rym", "rzm")


def bounds(name, im, jm, lm, nt=1):
    """The declared (lower, upper) bounds of a state array."""
    cells = [(-1, im + 2), (-1, jm + 2)]
    faces = [(0, im + 1), (0, jm + 1), (0, lm + 1)]
    table = {
        "m": [*cells, (1, lm)],
        "am": faces, "bm": faces, "cm": faces,
        "pu": [(0, im), (1, jm), (1, lm)],
        "pv": [(1, im), (1, jm + 1), (1, lm)],
        "sp": [*cells, (1, 1)],
        "phlb": [*cells, (1, lm + 1)],
        "dxyp": [(1, jm)],
    }  # fmt: skip
    for q in TRACERS:
        table[q] = [*cells, (1, lm), (1, nt)]
    return table[name]
