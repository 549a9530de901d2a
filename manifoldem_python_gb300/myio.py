"""Pickle dictionary I/O with the reference's format (``modules/myio.py:21-51``): one dict per
file, protocol ``pickle.HIGHEST_PROTOCOL``; a file that fails to unpickle reads as None."""
import pickle


def fin1(filename):
    with open(filename, 'rb') as f:
        try:
            return pickle.load(f)
        except Exception:
            return None


def fout1(filename, key_list, v_list):
    to_save = dict((key_list[i], v_list[i]) for i in range(len(key_list)))
    with open(filename, 'wb') as f:
        pickle.dump(to_save, f, protocol=pickle.HIGHEST_PROTOCOL)


def fout2(filename, d):
    fout1(filename, list(d.keys()), list(d.values()))
