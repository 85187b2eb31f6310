// Empty stand-in: the reference force laws are compiled as host code here.
#pragma once
