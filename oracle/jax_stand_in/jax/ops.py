from ._missing import missing_attr


def __getattr__(name):
    return missing_attr('ops.' + name, placeholder=True)
