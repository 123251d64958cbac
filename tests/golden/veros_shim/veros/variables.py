class Variable:
    def __init__(self, name, dims, units="", long_description="", **kwargs):
        self.name = name
        self.dims = dims
        self.units = units
