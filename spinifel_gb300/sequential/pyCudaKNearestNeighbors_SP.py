"""Single-precision KNN module, drop-in for the pybind11 module built from
spinifel/sequential/orientation_matching_sp.cu (PYBIND11_MODULE at :732)."""
import numpy as np

from ._knn_module import euclidean_distance, heap_sort


def cudaEuclideanDistance(refImgs, dataImgs, numRefImgs, numDataImgs, totalPixels, deviceId):
    return euclidean_distance(np.float32, refImgs, dataImgs, numRefImgs, numDataImgs,
                              totalPixels, deviceId)


def cudaHeapSort(euDist, numDataImgs, numRefImgs, totalPixels, totalNN, deviceId):
    return heap_sort(np.float32, euDist, numDataImgs, numRefImgs, totalPixels, totalNN, deviceId)
