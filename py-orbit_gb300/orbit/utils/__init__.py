"""Utility classes (py/orbit/utils/__init__.py)."""


class OrbitFinalizeError(RuntimeError):
    """Raised where the reference calls orbitFinalize (which exits)."""


def orbitFinalize(message=None):
    """The reference prints the message and exits the process
    (py/orbit/utils/orbitFinalize.py); here the error is raised instead."""
    raise OrbitFinalizeError(message or "orbitFinalize")


class NamedObject:
    """An object with a name (py/orbit/utils/NamedObject.py)."""

    def __init__(self, name="no name"):
        self.__name = name

    def setName(self, name="no name"):
        self.__name = name

    def getName(self):
        return self.__name


class TypedObject:
    """An object with a type (py/orbit/utils/TypedObject.py)."""

    def __init__(self, type_in="no type"):
        self.__type = type_in

    def setType(self, type_in="no type"):
        self.__type = type_in

    def getType(self):
        return self.__type


class ParamsDictObject:
    """An object with a parameters dictionary (py/orbit/utils/ParamsDictObject.py)."""

    def __init__(self):
        self.__paramsDict = {}

    def addParam(self, key, value):
        self.__paramsDict[key] = value

    def removeParam(self, key):
        self.__paramsDict.pop(key, None)

    def setParam(self, key, value):
        self.__paramsDict[key] = value

    def setParamsDict(self, params):
        self.__paramsDict = params

    def updateParamsDict(self, params):
        self.__paramsDict.update(params)

    def getParamsDict(self):
        return self.__paramsDict

    def hasParam(self, key):
        return key in self.__paramsDict

    def getParam(self, key):
        return self.__paramsDict[key]


speed_of_light = 2.99792458e+8

__all__ = ["orbitFinalize", "OrbitFinalizeError", "NamedObject", "TypedObject", "ParamsDictObject",
           "speed_of_light"]
