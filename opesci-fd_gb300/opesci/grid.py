"""Grid base: generate / compile / execute / convergence (placeholder, filled below)."""


class Grid(object):
    src_code = None
    src_file = None
    src_lib = None
    _library = None
    _arg_grid = None
    _arg_conv = None

    def __init__(self):
        pass
