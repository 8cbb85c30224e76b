from .build import build

build()
