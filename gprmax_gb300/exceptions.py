"""Error types raised by the input front-end and the solver (``gprMax/exceptions.py:29-46``)."""


class GeneralError(ValueError):
    """Raised for errors that are not specific to one input command."""

    def __init__(self, message, *args):
        self.message = message
        super().__init__(message, *args)


class CmdInputError(ValueError):
    """Raised for an invalid input command or parameter."""

    def __init__(self, message, *args):
        self.message = message
        super().__init__(message, *args)


class SolverError(RuntimeError):
    """Raised when the native GB300 solver returns an error status."""
