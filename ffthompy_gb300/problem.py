"""Problem definition and dispatch, mirroring ffthompy/problem.py.

Problem(conf_problem, conf) parses one entry of an input file's `problems`
list (problem.py:9-68); calculate() runs applications.<physics>
(problem.py:70-83); postprocessing() prints and optionally pickles the
output (problem.py:85-126).  Keys are compared with == (the reference's
`is` comparisons only work for interned literals).
"""
import os
import pickle
import sys
import time

import numpy as np

from . import applications


class Problem:
    def __init__(self, conf_problem=None, conf=None):
        self.__dict__.update(conf_problem)
        if isinstance(self.material, str):
            conf_material = conf.materials[self.material]
        else:
            conf_material = self.material
        self.material = self.parse_material(conf_material)
        self.Y = np.array(self.material['Y'], dtype=np.float64)
        self.dim = self.Y.size
        if self.physics == 'scalar':
            self.shape = (self.dim,)
        elif self.physics == 'elasticity':
            self.shape = (self.dim * (self.dim + 1) // 2,)
        self.output = {}

    @staticmethod
    def parse_material(conf_material):
        if 'fun' in conf_material:
            return conf_material
        incl = list(conf_material['inclusions'])
        for key in ('all', 'otherwise'):
            n = incl.count(key)
            if n > 1:
                raise ValueError("Maximal one occurrence of inclusion 'otherwise' or 'all' "
                                 "is allowed!")
            if n == 1 and incl.index(key) != len(incl) - 1:
                raise ValueError('inclusion ("all" or "otherwise") has to be at the end of '
                                 'the list')
        return conf_material

    def calculate(self):
        t0 = time.time()
        fn = getattr(applications, self.physics, None)
        if fn is None:
            raise NotImplementedError('Not implemented physics ({0}).'.format(self.physics))
        fn(self)
        self.output.setdefault('time', {})['calculate'] = time.time() - t0

    def postprocessing(self):
        output = self.output
        if self.physics in ('scalar', 'elasticity'):
            print('\nHomogenized matrices')
            for pd in self.solve['primaldual']:
                for key, val in output['mat_' + pd].items():
                    print(key)
                    print(val)
        if hasattr(self, 'save'):
            # the reference's layout (problem.py:98-126): self.output with the
            # problem's definition added - mat_<pd> dicts of arrays, sol_<pd>
            # lists of Tensors (values pickled as host arrays), res_<pd> lists
            # of {'cb': CallBack, 'info': {...}}
            self.save.setdefault('data', 'all')
            data = dict(self.output)
            material = {}
            for k, v in self.material.items():
                try:
                    pickle.dumps(v, protocol=3)
                except Exception:       # e.g. a 'fun' defined in a closure
                    continue
                material[k] = v
            data.update({'physics': self.physics, 'solve': self.solve, 'solver': self.solver,
                         'postprocess': self.postprocess, 'save': self.save,
                         'material': material})
            filename = self.save['filename']
            dirs = os.path.dirname(filename)
            if dirs and not os.path.exists(dirs):
                os.makedirs(dirs)
            with open(filename, 'wb') as fop:
                pickle.dump(data, fop, protocol=3)

    def __repr__(self):
        ss = 'Class : {}\n'.format(self.__class__.__name__)
        ss += '    name : {}\n    physics = {}\n    dim = {} (dimension)\n'.format(
            self.name, self.physics, self.dim)
        ss += '    Y = {} (PUC size)\n'.format(self.Y)
        return ss


def import_file(file_name):
    """Import an input file as a module (problem.py:143-160)."""
    module_path = os.path.dirname(os.path.abspath(file_name))
    added = module_path not in sys.path
    if added:
        sys.path.insert(0, module_path)
    try:
        conf = __import__(os.path.splitext(os.path.basename(file_name))[0])
    finally:
        if added:
            sys.path.remove(module_path)
    return conf
