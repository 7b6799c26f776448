class StaggeredCudaTemplate(object):
    def __init__(self, grid):
        self.grid = grid
