import numpy as np


def relu(x):
    return np.maximum(x, 0)
