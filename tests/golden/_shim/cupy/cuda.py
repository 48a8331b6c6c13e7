"""``cupy.cuda`` stand-in: a stream whose captures record and whose graphs replay."""

_CAPTURE = []  # stack of lists; the top one receives launches while capturing


def _capture_list():
    return _CAPTURE[-1] if _CAPTURE else None


class _Graph:
    def __init__(self, calls):
        self.calls = calls

    def upload(self, stream=None):
        pass

    def launch(self, stream=None):
        for fn, args in self.calls:
            fn(*args)


class Stream:
    null = None  # set below

    def __init__(self, non_blocking=False):
        pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False

    def synchronize(self):
        pass

    def begin_capture(self):
        _CAPTURE.append([])

    def end_capture(self):
        return _Graph(_CAPTURE.pop())


Stream.null = Stream()
