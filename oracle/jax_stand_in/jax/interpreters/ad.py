from .._missing import missing_attr


def __getattr__(name):
    return missing_attr('interpreters.ad.' + name, placeholder=True)
