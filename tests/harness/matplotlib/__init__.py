"""matplotlib stand-in (test infrastructure): accepts every call the
reference's harness makes for its diagnostic figures and draws nothing."""


class _Anything:
    def __getattr__(self, name):
        return _Anything()

    def __call__(self, *args, **kwargs):
        return _Anything()

    def __getitem__(self, key):
        return _Anything()

    def __iter__(self):
        return iter(())


def use(*args, **kwargs):
    pass


def __getattr__(name):
    return _Anything()
