class _Isotope:
    def __init__(self, mass_number, mass):
        self.mass_number = mass_number
        self.mass = mass


class element:
    _table = {
        "C": (12.011, [(12, 12.0)]),
        "O": (15.999, [(16, 15.99491461957)]),
        "S": (32.06, [(32, 31.9720711744)]),
        "H": (1.008, [(1, 1.00782503223)]),
    }

    def __init__(self, symbol):
        self.mass, iso = self._table[symbol]
        self.isotopes = [_Isotope(n, m) for n, m in iso]
