class Setting:
    def __init__(self, default, type, description=""):
        self.default = default
        self.type = type
        self.description = description
