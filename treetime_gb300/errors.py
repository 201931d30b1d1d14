"""Exception types of the TreeTime API, kept with the same names and hierarchy
so that callers catching them keep working (treetime/__init__.py:8-40)."""


class TreeTimeError(Exception):
    """Incorrect use of the API or input that violates its assumptions."""


class MissingDataError(TreeTimeError):
    """Tree or alignment missing, or too few sequences match the tree."""


class UnknownMethodError(TreeTimeError):
    """An unknown reconstruction or branch-length method was requested."""


class NotReadyError(TreeTimeError):
    """Results were requested before the inference that produces them ran."""


class TreeTimeUnknownError(Exception):
    """Inference failed for a reason that was not anticipated."""


class DeviceError(TreeTimeError):
    """The CUDA library reported a failure (status code and message attached)."""

    def __init__(self, status, message):
        super().__init__("%s (status %d)" % (message, status))
        self.status = status
