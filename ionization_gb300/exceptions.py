"""Exception types, same names and hierarchy as ionization/exceptions.py:1-40."""


class IonizationException(Exception):
    pass


class InvalidPotentialParameter(IonizationException):
    pass


class InvalidMaskParameter(IonizationException):
    pass


class IllegalQuantumState(IonizationException):
    """Attempt to construct a state with an illegal quantum number."""


class InvalidQuantumStateParameter(IonizationException):
    pass


class InvalidChoice(IonizationException):
    pass


class InvalidWrappingDirection(IonizationException):
    pass


class MissingDatastore(IonizationException):
    pass


class UnknownData(IonizationException):
    pass


class DuplicateDatastores(IonizationException):
    pass


class UnsupportedMesh(IonizationException):
    """The requested mesh / operator / method combination has no device path."""
