"""No-op ``matplotlib.pyplot`` stand-in (test infrastructure only)."""


def __getattr__(name):
    def _noop(*args, **kwargs):
        return None

    return _noop
