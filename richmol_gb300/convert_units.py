"""Unit conversion factors used on the propagation path, from CODATA values in
scipy.constants (same definitions as richmol/convert_units.py:5-110)."""
from scipy import constants


def J_to_invcm():
    """Joule -> cm^-1."""
    return 1.0 / (constants.value("Planck constant") * 1e2 * constants.value("speed of light in vacuum"))


def MHz_to_invcm():
    """MHz -> cm^-1."""
    return 1.0 / constants.value("speed of light in vacuum") * 1e4


def AUdip_x_Vm_to_invcm():
    """dipole (atomic units) x field (V/m) -> cm^-1."""
    return constants.value("atomic unit of electric dipole mom.") / (
        constants.value("Planck constant") * constants.value("speed of light in vacuum")) / 1e2


def AUpol_x_Vm_to_invcm():
    """polarizability (atomic units) x field^2 (V^2/m^2) -> cm^-1."""
    return constants.value("atomic unit of electric polarizability") / (
        constants.value("Planck constant") * constants.value("speed of light in vacuum")) / 1e2
