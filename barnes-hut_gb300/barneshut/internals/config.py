"""Process-global INI configuration (python-bh/barneshut/internals/config.py:8-29).

Same interface: ``Config.read_file(path)`` then ``Config.get(section, key)``.
Without ``read_file`` the package's ``configs/default.ini`` is used.
"""
from configparser import ConfigParser
from pathlib import Path

configs_dir = Path(__file__).resolve().parent.parent.parent / "configs"


class Config:

    def __init__(self, ini_path=None):
        self.parser = ConfigParser()
        self.parser.read(ini_path if ini_path is not None else configs_dir / "default.ini")

    @staticmethod
    def read_file(ini_path):
        global config_instance
        config_instance = Config(ini_path)

    @staticmethod
    def _inst():
        global config_instance
        if config_instance is None:
            config_instance = Config()
        return config_instance

    @staticmethod
    def get(*args, **kwargs):
        return Config._inst().parser.get(*args, **kwargs)

    @staticmethod
    def getint(*args, **kwargs):
        return Config._inst().parser.getint(*args, **kwargs)

    @staticmethod
    def getfloat(*args, **kwargs):
        return Config._inst().parser.getfloat(*args, **kwargs)

    @staticmethod
    def getboolean(*args, **kwargs):
        return Config._inst().parser.getboolean(*args, **kwargs)


config_instance = None
