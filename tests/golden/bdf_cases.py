"""Synthetic Nastran bulk-data decks for the BDF loader fixtures.

mixed_deck()     every card form the loader reads: GRID in small fixed, free
                 (comma) and large (GRID*) fields with the Nastran real forms
                 (1.5-3, -2.+1, 1.0D-2, 3.E+0), element cards in small and
                 large fields with continuation lines (CQUAD4, CQUAD4*,
                 CQUADR, CQUAD9, CTRIA3, CBAR, CHEXA, CTETRA with 4 and 10
                 nodes), SPC and SPC*, comment and component-name lines,
                 cards the loader skips, unsorted and gapped node and
                 element numbers, and text after ENDDATA.
plain_deck()     the whole file as bulk data (no BEGIN BULK, no ENDDATA),
                 CRLF line ends.
crlf_continuation_deck()
                 CRLF line ends under a continued card: a deck the
                 reference's loader rejects.
cylinder_deck()  a Quad4 cylinder as GRID* / CQUAD4 cards (nodes and
                 elements written in shuffled order), clamped at x = 0 and
                 compressed by a prescribed axial displacement at x = L
                 (two SPC cards per loaded node, as displacement control).

Every line carries all the columns the loader reads, so the decks exercise
the loader's documented field layout only.
"""
from __future__ import annotations

import numpy as np


def _small(name, *fields):
    s = f"{name:<8}" + "".join(f"{str(f):>8}" for f in fields)
    return s


def _wide(name, *fields):
    return f"{name:<8}" + "".join(f"{str(f):>16}" for f in fields)


def mixed_deck() -> str:
    L = []
    L.append("$ synthetic deck for the BDF loader")
    L.append("SOL 105")
    L.append("CEND")
    L.append("TITLE = LOADER CARDS")
    L.append("BEGIN BULK")
    L.append(f"{'$       Shell element data for family':<41}SKIN")
    L.append(f"{'$       Shell element data for family':<41}SPAR web")
    L.append("$ comment line inside the bulk data")
    # small-field GRIDs (node, cp, x, y, z), Nastran real forms
    L.append(_small("GRID", 7, 0, "1.5-3", "-2.+1", "1.0D-2"))
    L.append(_small("GRID", 3, "", "3.E+0", ".25", "-0.5"))
    L.append(_small("GRID", 12, 0, "7.", "1.25+0", "-4.-1"))
    L.append(_small("GRID", 1, 0, "0.0", "0.0", "0.0"))
    L.append(_small("GRID", 2, 0, "1.0", "0.0", "0.0"))
    L.append(_small("GRID", 4, 0, "0.0", "1.0", "0.0"))
    L.append(_small("GRID", 5, 0, "1.0", "1.0", "0.0"))
    # free-field GRIDs (comma separated after the card name field)
    L.append("GRID    6,0,2.0,0.5,0.125")
    L.append("GRID    8,0,-1.5,2.5,3.5")
    L.append("GRID    9,,2.5E-1,1.D0,-7.5")
    # large-field GRIDs: node 8-24, cp 24-40, x 40-56, y 56-72; z on line 2
    L.append(_wide("GRID*", 10, 0, "1.234567890123", "-4.5E-01") + "*G10")
    L.append(f"{'*G10':<8}{'2.000000000001':>16}")
    L.append(_wide("GRID*", 11, "", "-3.25", "6.5+1") + "*G11")
    L.append(f"{'*G11':<8}{'-1.0D-3':>16}")
    for k in range(13, 31):
        L.append(_small("GRID", 100 + k, 0, f"{0.1 * k:.2f}", f"{0.05 * k:.3f}", f"{-0.02 * k:.3f}"))
    # cards the loader does not read
    L.append(_small("PSHELL", 1, 1, "0.01", 1))
    L.append(_small("MAT1", 1, "7.+10", "", "0.3"))
    # elements: numbers out of order, components 1..7
    L.append(_small("CQUAD4", 40, 1, 1, 2, 5, 4))
    L.append(_small("CQUADR", 12, 1, 2, 6, 8, 5))
    L.append(_wide("CQUAD4*", 25, 1, 4, 5))
    L.append(f"{'*':<8}{9:>16}{3:>16}")
    L.append(_small("CQUAD9", 33, 2, 1, 2, 5, 4, 6, 7))
    L.append(f"{'':<8}{8:>8}{9:>8}{10:>8}")
    L.append(_small("CTRIA3", 5, 3, 11, 12, 3))
    L.append(_small("CBAR", 7, 4, 113, 114, "0.0", "1.0", "0.0"))
    L.append(_small("CHEXA", 50, 5, 113, 114, 115, 116, 117, 118))
    L.append(f"{'':<8}{119:>8}{120:>8}")
    L.append(_small("CTETRA", 41, 6, 121, 122, 123, 124))
    L.append(_small("CTETRA", 42, 7, 121, 122, 123, 124, 125, 126))
    L.append(f"{'':<8}{127:>8}{128:>8}{129:>8}{130:>8}")
    L.append(_small("CQUAD4", 2, 3, 3, 7, 12, 11))
    # single-point constraints: small (node 16-24, dofs 24-32, value 32-40)
    L.append(_small("SPC", 1, 1, "123456", "0.0"))
    L.append(_small("SPC", 1, 12, "135", "-1.-5"))
    L.append(_small("SPC", 1, 2, "2", "2.5-3"))
    # large (node 24-40, dofs 40-56, value 56-72)
    L.append(_wide("SPC*", 1, 10, "456", "-1.E-5"))
    L.append(_wide("SPC*", 2, 128, "78", "3.5"))
    L.append("ENDDATA")
    L.append("GRID           999       0     9.0     9.0     9.0")
    return "\n".join(L) + "\n"


def plain_deck() -> str:
    """No executive/case sections and no BEGIN BULK (the whole file is bulk
    data), CRLF line ends, no ENDDATA, one-line element cards and a trailing
    comment."""
    L = []
    for k in range(1, 10):
        L.append(_small("GRID", 10 * k, 0, f"{(k - 1) % 3}.", f"{(k - 1) // 3}.", "0."))
    L.append(_small("CQUAD4", 3, 2, 10, 20, 50, 40))
    L.append(_small("CQUAD4", 1, 2, 20, 30, 60, 50))
    L.append(_small("CTRIA3", 2, 1, 40, 50, 80))
    L.append(_small("SPC", 3, 10, "123", "1.5-2"))
    L.append("$ end of deck")
    return "\r\n".join(L) + "\r\n"


def crlf_continuation_deck() -> str:
    """CRLF line ends under a card that continues: the "\r" ending the first
    line is read as a node field of 0, so the card ends there and has too few
    nodes (the reference's loader aborts on this deck)."""
    L = [_small("GRID", k, 0, f"{k}.", "0.", "0.") for k in range(1, 10)]
    L.append(_small("CQUAD9", 1, 1, 1, 2, 3, 4, 5, 6))
    L.append(f"{'':<8}{7:>8}{8:>8}{9:>8}")
    return "\r\n".join(L) + "\r\n"


def cylinder_deck(m, disp=-1.0e-5, seed=5):
    """Deck for ShellMesh m (Quad4): GRID* with 10 significant digits,
    CQUAD4 in Nastran cyclic order, SPC 123456 on the x = 0 ring, SPC 23
    (0.0) and SPC 1 (disp) on the x = L ring."""
    rng = np.random.default_rng(seed)
    X, conn = m.X, m.conn
    nn, ne = X.shape[0], conn.shape[0]
    L = ["$ synthetic cylinder deck", "BEGIN BULK"]
    for i in rng.permutation(nn):
        L.append(_wide("GRID*", i + 1, 0, f"{X[i, 0]:16.9E}", f"{X[i, 1]:16.9E}") + f"*N{i + 1}")
        L.append(f"{'*N' + str(i + 1):<8}{X[i, 2]:16.9E}")
    for e in rng.permutation(ne):
        c = conn[e]
        L.append(_small("CQUAD4", e + 1, 1, c[0] + 1, c[1] + 1, c[3] + 1, c[2] + 1))
    x = X[:, 0]
    for i in np.where(np.abs(x) < 1e-12)[0]:
        L.append(_small("SPC", 1, i + 1, "123456", "0.0"))
    for i in np.where(np.abs(x - x.max()) < 1e-12)[0]:
        L.append(_small("SPC", 1, i + 1, "23", "0.0"))
        L.append(_small("SPC", 1, i + 1, "1", f"{disp:.1E}"))
    L.append("ENDDATA")
    return "\n".join(L) + "\n"
