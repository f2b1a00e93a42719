from .._missing import missing_attr


def __getattr__(name):
    return missing_attr('image.' + name, placeholder=True)
