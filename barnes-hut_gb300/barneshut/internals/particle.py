"""Field indices of the N x 10 float64 particle record
(python-bh/barneshut/internals/particle.py:3-15)."""
import numpy as np

px, py = 0, 1
mass = 2
vx, vy = 3, 4
ax, ay = 5, 6
gx, gy = 7, 8
pid = 9

gxf, gyf = "f7", "f8"
massf = "f2"
idf = "f9"
nfields = 10
fieldsstr = "f8,f8,f8,f8,f8,f8,f8,f8,f8,f8"
ftype = np.float64
