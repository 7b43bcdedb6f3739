"""Test-only stand-in for the ``xraylib`` element tables, used only when generating the golden fixtures.

The reference imports ``xraylib`` at module level for element symbols, densities and atomic weights of its material
catalogue. The fixtures use the synthetic cross-section library, which never reads those values, so placeholder numbers
are enough to make the package importable. This module is never imported by the product or by the tests.
"""

_SYMBOLS = ("H He Li Be B C N O F Ne Na Mg Al Si P S Cl Ar K Ca Sc Ti V Cr Mn Fe Co Ni Cu Zn Ga Ge As Se Br Kr Rb Sr "
            "Y Zr Nb Mo Tc Ru Rh Pd Ag Cd In Sn Sb Te I Xe Cs Ba La Ce Pr Nd Pm Sm Eu Gd Tb Dy Ho Er Tm Yb Lu Hf Ta W "
            "Re Os Ir Pt Au Hg Tl Pb Bi Po At Rn Fr Ra Ac Th Pa U Np Pu Am Cm Bk Cf").split()

K_SHELL = 0


def AtomicNumberToSymbol(Z):
    return _SYMBOLS[int(Z) - 1]


def SymbolToAtomicNumber(symbol):
    return _SYMBOLS.index(symbol) + 1


def ElementDensity(Z):
    return 1.0


def AtomicWeight(Z):
    return 2.0 * float(Z)
